// cg_sample.cuh -- device-side sampling of the mip pyramid, the hash-noise fBm
// and the sun cone, shared by the trace kernels.
#pragma once

#include <cuda_fp16.h>

#include "cg_internal.h"

#define CG_MAX_SUN_STEPS 64

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

namespace cgs {

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float fp16_hi(uint32_t v) {
    return __half2float(__ushort_as_half((unsigned short)(v >> 16)));
}

// Trilinear at level l of channel R (and G when WANT_G), level-0 voxel-space
// position (px,py,pz).  BORDER: taps outside the level read 0; otherwise
// clamp to edge.  Texel coordinates x = p * N_l / D - 0.5.
template <int FMT, bool WANT_G, bool BORDER>
__device__ __forceinline__ float2 tri(const VolDesc& vd, int l, float px, float py, float pz) {
    const int N = vd.dims[l];
    const float sc = (float)N / (float)vd.D;
    float x = px * sc - 0.5f, y = py * sc - 0.5f, z = pz * sc - 0.5f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float wx = x - fx, wy = y - fy, wz = z - fz;
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    int xs[2] = {ix, ix + 1}, ys[2] = {iy, iy + 1}, zs[2] = {iz, iz + 1};
    bool vx[2], vy[2], vz[2];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        vx[a] = (xs[a] >= 0 && xs[a] < N);
        vy[a] = (ys[a] >= 0 && ys[a] < N);
        vz[a] = (zs[a] >= 0 && zs[a] < N);
        xs[a] = min(max(xs[a], 0), N - 1);
        ys[a] = min(max(ys[a], 0), N - 1);
        zs[a] = min(max(zs[a], 0), N - 1);
    }
    float r[2][2][2], g[2][2][2];
    const long long base = vd.offs[l];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const long long idx = base + ((long long)zs[c] * N + ys[b]) * N + xs[a];
                const bool ok = !BORDER || (vx[a] && vy[b] && vz[c]);
                float rv = 0.f, gv = 0.f;
                if (FMT == 0) {
                    const float4* p4 = reinterpret_cast<const float4*>(vd.pyr);
                    if (WANT_G) {
                        float2 t = __ldg(reinterpret_cast<const float2*>(p4 + idx));
                        rv = t.x;
                        gv = t.y;
                    } else {
                        rv = __ldg(reinterpret_cast<const float*>(p4 + idx));
                    }
                } else {
                    uint32_t t = __ldg(reinterpret_cast<const uint32_t*>(vd.pyr) + idx);
                    rv = bf16_lo(t);
                    if (WANT_G) gv = fp16_hi(t);
                }
                r[c][b][a] = ok ? rv : 0.f;
                g[c][b][a] = ok ? gv : 0.f;
            }
    float2 out;
    {
        float x00 = r[0][0][0] + wx * (r[0][0][1] - r[0][0][0]);
        float x10 = r[0][1][0] + wx * (r[0][1][1] - r[0][1][0]);
        float x01 = r[1][0][0] + wx * (r[1][0][1] - r[1][0][0]);
        float x11 = r[1][1][0] + wx * (r[1][1][1] - r[1][1][0]);
        float y0 = x00 + wy * (x10 - x00);
        float y1 = x01 + wy * (x11 - x01);
        out.x = y0 + wz * (y1 - y0);
    }
    out.y = 0.f;
    if (WANT_G) {
        float x00 = g[0][0][0] + wx * (g[0][0][1] - g[0][0][0]);
        float x10 = g[0][1][0] + wx * (g[0][1][1] - g[0][1][0]);
        float x01 = g[1][0][0] + wx * (g[1][0][1] - g[1][0][0]);
        float x11 = g[1][1][0] + wx * (g[1][1][1] - g[1][1][0]);
        float y0 = x00 + wy * (x10 - x00);
        float y1 = x01 + wy * (x11 - x01);
        out.y = y0 + wz * (y1 - y0);
    }
    return out;
}

// Quadrilinear (GL_LINEAR_MIPMAP_LINEAR): lod clamped to [0, L-1].
template <int FMT, bool WANT_G, bool BORDER>
__device__ __forceinline__ float2 quad(const VolDesc& vd, float px, float py, float pz,
                                       float lod) {
    const float maxl = (float)(vd.L - 1);
    lod = fminf(fmaxf(lod, 0.f), maxl);
    const int l0 = (int)floorf(lod);
    const float fr = lod - (float)l0;
    float2 a = tri<FMT, WANT_G, BORDER>(vd, l0, px, py, pz);
    if (fr > 0.f && l0 + 1 < vd.L) {
        float2 b = tri<FMT, WANT_G, BORDER>(vd, l0 + 1, px, py, pz);
        a.x = a.x + fr * (b.x - a.x);
        a.y = a.y + fr * (b.y - a.y);
    }
    return a;
}

// Same with a precomputed (l0, frac) split.
template <int FMT, bool WANT_G, bool BORDER>
__device__ __forceinline__ float2 quad_split(const VolDesc& vd, float px, float py, float pz,
                                             int l0, float fr) {
    float2 a = tri<FMT, WANT_G, BORDER>(vd, l0, px, py, pz);
    if (fr > 0.f && l0 + 1 < vd.L) {
        float2 b = tri<FMT, WANT_G, BORDER>(vd, l0 + 1, px, py, pz);
        a.x = a.x + fr * (b.x - a.x);
        a.y = a.y + fr * (b.y - a.y);
    }
    return a;
}

// Neumaier compensated accumulation.
__device__ __forceinline__ void neumaier(float& sum, float& comp, float term) {
    float t = sum + term;
    if (fabsf(sum) >= fabsf(term))
        comp += (sum - t) + term;
    else
        comp += (term - t) + sum;
    sum = t;
}

// Sun cone from level-0 voxel-space position v toward unit direction s.
// Mode 0 returns optical depth (world units); mode 1 the reference's
// weighted sum of the light channel.
template <int FMT>
__device__ __forceinline__ float sun_cone(const VolDesc& vd, const ConeSchedule& cs, float vx,
                                          float vy, float vz, float sx, float sy, float sz) {
    if (cs.mode == 1) {
        float acc = 0.f;
        for (int i = 0; i < cs.steps; ++i) {
            float h = cs.h[i];
            float2 c = quad_split<FMT, true, false>(vd, vx + h * sx, vy + h * sy, vz + h * sz,
                                                    cs.l0[i], cs.frac[i]);
            acc += c.y * cs.w[i];
        }
        return acc;
    }
    const float D = (float)vd.D, E = cs.edge;
    float tau = 0.f, comp = 0.f;
    for (int i = 0; i < cs.steps; ++i) {
        float h = cs.h[i];
        float x = vx + h * sx, y = vy + h * sy, z = vz + h * sz;
        if (x < -E || y < -E || z < -E || x > D + E || y > D + E || z > D + E) break;
        float2 c = quad_split<FMT, false, true>(vd, x, y, z, cs.l0[i], cs.frac[i]);
        neumaier(tau, comp, c.x * cs.w[i]);
    }
    return tau + comp;
}

// Number of samples the transmittance cone takes before leaving the box
// (statistics only).
__device__ __forceinline__ unsigned cone_samples(const VolDesc& vd, const ConeSchedule& cs,
                                                 float vx, float vy, float vz, float sx,
                                                 float sy, float sz) {
    if (cs.mode == 1) return (unsigned)cs.steps;
    const float D = (float)vd.D, E = cs.edge;
    unsigned n = 0;
    for (int i = 0; i < cs.steps; ++i) {
        float h = cs.h[i];
        float x = vx + h * sx, y = vy + h * sy, z = vz + h * sz;
        if (x < -E || y < -E || z < -E || x > D + E || y > D + E || z > D + E) break;
        n++;
    }
    return n;
}

// ---- hash value-noise fBm --------------------------------------------------

// PCG3D (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020).
__device__ __forceinline__ uint3 pcg3d(uint3 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.x += v.y * v.z;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.x ^= v.x >> 16;
    v.y ^= v.y >> 16;
    v.z ^= v.z >> 16;
    v.x += v.y * v.z;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    return v;
}

__device__ __forceinline__ float lattice(int ix, int iy, int iz, uint32_t k) {
    uint3 h = pcg3d(make_uint3((uint32_t)ix + k, (uint32_t)iy + (k ^ 0x68E31DA4u),
                               (uint32_t)iz + (k ^ 0xB5297A4Du)));
    return (float)(h.x >> 8) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ float value_noise(float x, float y, float z, uint32_t k) {
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float ux = x - fx, uy = y - fy, uz = z - fz;
    float wx = ux * ux * (3.f - 2.f * ux);
    float wy = uy * uy * (3.f - 2.f * uy);
    float wz = uz * uz * (3.f - 2.f * uz);
    float c000 = lattice(ix, iy, iz, k), c100 = lattice(ix + 1, iy, iz, k);
    float c010 = lattice(ix, iy + 1, iz, k), c110 = lattice(ix + 1, iy + 1, iz, k);
    float c001 = lattice(ix, iy, iz + 1, k), c101 = lattice(ix + 1, iy, iz + 1, k);
    float c011 = lattice(ix, iy + 1, iz + 1, k), c111 = lattice(ix + 1, iy + 1, iz + 1, k);
    float x00 = c000 + wx * (c100 - c000);
    float x10 = c010 + wx * (c110 - c010);
    float x01 = c001 + wx * (c101 - c001);
    float x11 = c011 + wx * (c111 - c011);
    float y0 = x00 + wy * (x10 - x00);
    float y1 = x01 + wy * (x11 - x01);
    return y0 + wz * (y1 - y0);
}

// fBm over world position p; octave key k = seed*0x9E3779B9 + o*0x85EBCA6B + 1.
__device__ __forceinline__ float fbm(const TraceParams& tp, float px, float py, float pz) {
    if (tp.noise_octaves <= 0) return 1.f;
    float amp = 1.f, sum = 0.f, f = tp.noise_freq;
    for (int o = 0; o < tp.noise_octaves; ++o) {
        uint32_t k = tp.noise_seed * 0x9E3779B9u + (uint32_t)o * 0x85EBCA6Bu + 1u;
        sum += amp * value_noise(px * f, py * f, pz * f, k);
        amp *= tp.noise_gain;
        f *= tp.noise_lac;
    }
    return sum * tp.noise_inv_norm;
}

}  // namespace cgs
