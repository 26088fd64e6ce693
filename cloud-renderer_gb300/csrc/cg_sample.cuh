// cg_sample.cuh -- device-side sampling of the mip pyramid, the hash-noise fBm
// and the sun cone, shared by the trace kernels.
#pragma once

#include <cuda_fp16.h>

#include "cg_internal.h"



namespace cgs {

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float fp16_hi(uint32_t v) {
    return __half2float(__ushort_as_half((unsigned short)(v >> 16)));
}

// One voxel's (R, G) at flat index idx.
template <int FMT, bool WANT_G>
__device__ __forceinline__ float2 fetch(const void* pyr, int idx) {
    if (FMT == 0) {
        const float4* p4 = reinterpret_cast<const float4*>(pyr);
        if (WANT_G) return __ldg(reinterpret_cast<const float2*>(p4 + idx));
        return make_float2(__ldg(reinterpret_cast<const float*>(p4 + idx)), 0.f);
    }
    uint32_t t = __ldg(reinterpret_cast<const uint32_t*>(pyr) + idx);
    return make_float2(bf16_lo(t), WANT_G ? fp16_hi(t) : 0.f);
}

// fetch() at a flat index of the whole pyramid, checked in the bounds-check
// build (an index past the last level reads 0).
template <int FMT, bool WANT_G>
__device__ __forceinline__ float2 fetch_vd(const VolDesc& vd, int idx) {
    if (!CG_IN_BOUNDS(idx, vd.nvox)) return make_float2(0.f, 0.f);
    return fetch<FMT, WANT_G>(vd.pyr, idx);
}

__device__ __forceinline__ float lerp3(const float c[8], float wx, float wy, float wz) {
    float x00 = c[0] + wx * (c[1] - c[0]);
    float x10 = c[2] + wx * (c[3] - c[2]);
    float x01 = c[4] + wx * (c[5] - c[4]);
    float x11 = c[6] + wx * (c[7] - c[6]);
    float y0 = x00 + wy * (x10 - x00);
    float y1 = x01 + wy * (x11 - x01);
    return y0 + wz * (y1 - y0);
}

// Occupancy of the level-l brick holding texel (ix, iy, iz) (see VolDesc).
__device__ __forceinline__ bool occupied(const VolDesc& vd, int l, int ix, int iy, int iz) {
    const int nb = vd.occ_nb[l], sh = vd.occ_shift;
    int bx = min(max(ix >> sh, 0), nb - 1);
    int by = min(max(iy >> sh, 0), nb - 1);
    int bz = min(max(iz >> sh, 0), nb - 1);
    const int at = vd.occ_off[l] + (bz * nb + by) * nb + bx;
    if (!CG_IN_BOUNDS(at, vd.occ_total)) return false;
    return __ldg(vd.occ + at) != 0;
}

// Trilinear at level l of channel R (and G when WANT_G), level-0 voxel-space
// position (px,py,pz).  BORDER: taps outside the level read 0; otherwise
// clamp to edge.  Texel coordinates x = p * N_l / D - 0.5.  SKIP_EMPTY: when
// the footprint's brick is unoccupied the result is exactly (0, 0) for R and
// is returned without touching the volume (callers that use G only where
// R > 0).
template <int FMT, bool WANT_G, bool BORDER, bool SKIP_EMPTY>
__device__ __forceinline__ float2 tri(const VolDesc& vd, int l, float px, float py, float pz) {
    const int N = vd.dims[l];
    const float sc = vd.lsc[l];  // N_l / D
    float x = px * sc - 0.5f, y = py * sc - 0.5f, z = pz * sc - 0.5f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float wx = x - fx, wy = y - fy, wz = z - fz;
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    if (SKIP_EMPTY && !occupied(vd, l, ix, iy, iz)) return make_float2(0.f, 0.f);
    float r[8], g[8];
    const int base = (int)vd.offs[l];
    if (ix >= 0 && iy >= 0 && iz >= 0 && ix + 1 < N && iy + 1 < N && iz + 1 < N) {
        // interior: one base index, fixed offsets
        const int i0 = base + (iz * N + iy) * N + ix;
        const int NN = N * N;
        const int o[8] = {0, 1, N, N + 1, NN, NN + 1, NN + N, NN + N + 1};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float2 t = fetch_vd<FMT, WANT_G>(vd, i0 + o[k]);
            r[k] = t.x;
            g[k] = t.y;
        }
    } else {
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
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int k = c * 4 + b * 2 + a;
                    const bool ok = !BORDER || (vx[a] && vy[b] && vz[c]);
                    float2 t = fetch_vd<FMT, WANT_G>(vd, base + (zs[c] * N + ys[b]) * N + xs[a]);
                    r[k] = ok ? t.x : 0.f;
                    g[k] = ok ? t.y : 0.f;
                }
    }
    return make_float2(lerp3(r, wx, wy, wz), WANT_G ? lerp3(g, wx, wy, wz) : 0.f);
}

// Quadrilinear with a precomputed (l0, frac) split.
template <int FMT, bool WANT_G, bool BORDER, bool SKIP_EMPTY>
__device__ __forceinline__ float2 quad_split(const VolDesc& vd, float px, float py, float pz,
                                             int l0, float fr) {
    float2 a = tri<FMT, WANT_G, BORDER, SKIP_EMPTY>(vd, l0, px, py, pz);
    if (fr > 0.f && l0 + 1 < vd.L) {
        float2 b = tri<FMT, WANT_G, BORDER, SKIP_EMPTY>(vd, l0 + 1, px, py, pz);
        a.x = a.x + fr * (b.x - a.x);
        a.y = a.y + fr * (b.y - a.y);
    }
    return a;
}

// Quadrilinear (GL_LINEAR_MIPMAP_LINEAR): lod clamped to [0, L-1].
template <int FMT, bool WANT_G, bool BORDER, bool SKIP_EMPTY>
__device__ __forceinline__ float2 quad(const VolDesc& vd, float px, float py, float pz,
                                       float lod) {
    const float maxl = (float)(vd.L - 1);
    lod = fminf(fmaxf(lod, 0.f), maxl);
    const int l0 = (int)floorf(lod);
    return quad_split<FMT, WANT_G, BORDER, SKIP_EMPTY>(vd, px, py, pz, l0, lod - (float)l0);
}

// ---- hardware-filtered sampling (surrogate renderer) ----------------------
// Same coordinates as tri(): the texture unit samples texel space at
// (p * N_l / D) with unnormalised coordinates, so its trilinear weights match
// the software path up to their 8-bit fixed-point precision; border
// addressing reads 0 outside the level.
template <bool SKIP_EMPTY>
__device__ __forceinline__ float2 tri_hw(const VolDesc& vd, int l, float px, float py, float pz) {
    const float sc = vd.lsc[l];  // N_l / D
    const float x = px * sc, y = py * sc, z = pz * sc;
    if (SKIP_EMPTY && !occupied(vd, l, (int)floorf(x - 0.5f), (int)floorf(y - 0.5f),
                                (int)floorf(z - 0.5f)))
        return make_float2(0.f, 0.f);
    return tex3D<float2>((cudaTextureObject_t)vd.tex[l], x, y, z);
}

template <bool SKIP_EMPTY>
__device__ __forceinline__ float2 quad_hw(const VolDesc& vd, float px, float py, float pz,
                                          float lod) {
    const float maxl = (float)(vd.L - 1);
    lod = fminf(fmaxf(lod, 0.f), maxl);
    const int l0 = (int)floorf(lod);
    const float fr = lod - (float)l0;
    float2 a = tri_hw<SKIP_EMPTY>(vd, l0, px, py, pz);
    if (fr > 0.f && l0 + 1 < vd.L) {
        float2 b = tri_hw<SKIP_EMPTY>(vd, l0 + 1, px, py, pz);
        a.x = a.x + fr * (b.x - a.x);
        a.y = a.y + fr * (b.y - a.y);
    }
    return a;
}

// View-march steps k (sample at t_k = tin + (k + 1/2) dt along the unit
// direction d from the eye) that can meet the occupied level-0 box (widened by
// one voxel, and by one step at either end): [k0, k1], empty (k0 > k1) when
// the ray misses it.  A step outside it whose sample has lod 0 reads exactly 0
// (its brick is unoccupied), so marches skip those steps.
__device__ __forceinline__ void occupied_steps(const VolDesc& vd, const float eye[3], float3 d,
                                               float tin, float dt, int Nv, int& k0, int& k1) {
    const int* b = vd.occ_box;
    const float D = (float)vd.D;
    const float dd[3] = {d.x, d.y, d.z};
    float ta = -1e30f, tb = 1e30f;
    k0 = Nv;
    k1 = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int lo = vd.D - __ldg(b + a), hi = __ldg(b + 3 + a);
        if (lo >= hi) return;  // nothing occupied
        const float vs = D / vd.range[a];
        const float ve = (eye[a] - vd.wmin[a]) * vs, dv = dd[a] * vs;
        const float l = (float)lo - 1.f, h = (float)hi + 1.f;
        if (dv == 0.f) {
            if (ve < l || ve > h) return;
            continue;
        }
        const float t0 = (l - ve) / dv, t1 = (h - ve) / dv;
        ta = fmaxf(ta, fminf(t0, t1));
        tb = fminf(tb, fmaxf(t0, t1));
    }
    if (!(tb >= ta)) return;
    const float fa = fmaxf((ta - tin) / dt - 0.5f, -1.f), fb = fminf((tb - tin) / dt - 0.5f, (float)Nv);
    k0 = max(0, (int)floorf(fa) - 1);
    k1 = min(Nv - 1, (int)ceilf(fb) + 1);
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
            float2 c = quad_split<FMT, true, false, false>(vd, vx + h * sx, vy + h * sy,
                                                           vz + h * sz, cs.l0[i], cs.frac[i]);
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
        float2 c = quad_split<FMT, false, true, true>(vd, x, y, z, cs.l0[i], cs.frac[i]);
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

__device__ __forceinline__ uint32_t octave_key(uint32_t seed, int o) {
    return seed * 0x9E3779B9u + (uint32_t)o * 0x85EBCA6Bu + 1u;
}

__device__ __forceinline__ float lattice(int ix, int iy, int iz, uint32_t k) {
    uint3 h = pcg3d(make_uint3((uint32_t)ix + k, (uint32_t)iy + (k ^ 0x68E31DA4u),
                               (uint32_t)iz + (k ^ 0xB5297A4Du)));
    return (float)(h.x >> 8) * (1.0f / 16777216.0f);
}

// Value noise of octave o at lattice coordinates (x, y, z): trilinear over
// the lattice with smoothstep weights.  Corner values come from the octave's
// table when the 2x2x2 corner block lies inside it, else from the hash.
__device__ __forceinline__ float value_noise(const TraceParams& tp, int o, float x, float y,
                                             float z) {
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float ux = x - fx, uy = y - fy, uz = z - fz;
    float wx = ux * ux * (3.f - 2.f * ux);
    float wy = uy * uy * (3.f - 2.f * uy);
    float wz = uz * uz * (3.f - 2.f * uz);
    float c[8];
    const int tx = ix - tp.nt.lo[o][0], ty = iy - tp.nt.lo[o][1], tz = iz - tp.nt.lo[o][2];
    const int dx = tp.nt.dim[o][0], dy = tp.nt.dim[o][1], dz = tp.nt.dim[o][2];
    if (tp.nt.tab && tx >= 0 && ty >= 0 && tz >= 0 && tx + 1 < dx && ty + 1 < dy && tz + 1 < dz) {
        const float* t = tp.nt.tab + tp.nt.off[o] + (tz * dy + ty) * dx + tx;
        const int sy = dx, sz = dx * dy;
        c[0] = __ldg(t);
        c[1] = __ldg(t + 1);
        c[2] = __ldg(t + sy);
        c[3] = __ldg(t + sy + 1);
        c[4] = __ldg(t + sz);
        c[5] = __ldg(t + sz + 1);
        c[6] = __ldg(t + sz + sy);
        c[7] = __ldg(t + sz + sy + 1);
    } else {
        const uint32_t k = octave_key(tp.noise_seed, o);
        c[0] = lattice(ix, iy, iz, k);
        c[1] = lattice(ix + 1, iy, iz, k);
        c[2] = lattice(ix, iy + 1, iz, k);
        c[3] = lattice(ix + 1, iy + 1, iz, k);
        c[4] = lattice(ix, iy, iz + 1, k);
        c[5] = lattice(ix + 1, iy, iz + 1, k);
        c[6] = lattice(ix, iy + 1, iz + 1, k);
        c[7] = lattice(ix + 1, iy + 1, iz + 1, k);
    }
    return lerp3(c, wx, wy, wz);
}

// Value noise by one hardware trilinear fetch: with i = floor(x) and w the
// smoothstep weights, the smoothstep-weighted blend of the 8 lattice values
// is the texture's linear filter at texel coordinate (i - lo) + w + 0.5.
__device__ __forceinline__ float value_noise_hw(const TraceParams& tp, int o, float x, float y,
                                                float z) {
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    int tx = (int)fx - tp.nt.lo[o][0], ty = (int)fy - tp.nt.lo[o][1], tz = (int)fz - tp.nt.lo[o][2];
    if (tp.nt.tex[o] && tx >= 0 && ty >= 0 && tz >= 0 && tx + 1 < tp.nt.dim[o][0] &&
        ty + 1 < tp.nt.dim[o][1] && tz + 1 < tp.nt.dim[o][2]) {
        float ux = x - fx, uy = y - fy, uz = z - fz;
        float wx = ux * ux * (3.f - 2.f * ux);
        float wy = uy * uy * (3.f - 2.f * uy);
        float wz = uz * uz * (3.f - 2.f * uz);
        return tex3D<float>((cudaTextureObject_t)tp.nt.tex[o], (float)tx + wx + 0.5f,
                            (float)ty + wy + 0.5f, (float)tz + wz + 0.5f);
    }
    return value_noise(tp, o, x, y, z);
}

// fBm at world position p: the noise domain is shifted by tp.noise_shift
// (q = p + shift; a zero shift leaves p unchanged).
__device__ __forceinline__ float fbm_hw(const TraceParams& tp, float px, float py, float pz) {
    if (tp.noise_octaves <= 0) return 1.f;
    px += tp.noise_shift[0];
    py += tp.noise_shift[1];
    pz += tp.noise_shift[2];
    float amp = 1.f, sum = 0.f, f = tp.noise_freq;
    for (int o = 0; o < tp.noise_octaves; ++o) {
        sum += amp * value_noise_hw(tp, o, px * f, py * f, pz * f);
        amp *= tp.noise_gain;
        f *= tp.noise_lac;
    }
    return sum * tp.noise_inv_norm;
}

// fBm from its precomputed volume (surrogate renderer): one hardware
// trilinear fetch at the noise coordinate q = p + shift; the volume holds fBm
// at its texel centres over the noise domain (NoiseTab.fbm_org / fbm_sc).
__device__ __forceinline__ float fbm_volume(const TraceParams& tp, float px, float py,
                                            float pz) {
    if (tp.noise_octaves <= 0) return 1.f;
    if (!tp.nt.fbm_tex) return fbm_hw(tp, px, py, pz);
    const float tx = (px + tp.noise_shift[0] - tp.nt.fbm_org[0]) * tp.nt.fbm_sc[0];
    const float ty = (py + tp.noise_shift[1] - tp.nt.fbm_org[1]) * tp.nt.fbm_sc[1];
    const float tz = (pz + tp.noise_shift[2] - tp.nt.fbm_org[2]) * tp.nt.fbm_sc[2];
    return tex3D<float>((cudaTextureObject_t)tp.nt.fbm_tex, tx, ty, tz);
}

// fBm = sum_o gain^o noise_o(q * freq * lac^o) / sum_o gain^o at the noise
// coordinate q (already shifted); 1 without octaves.
__device__ __forceinline__ float fbm_q(const TraceParams& tp, float qx, float qy, float qz) {
    if (tp.noise_octaves <= 0) return 1.f;
    float amp = 1.f, sum = 0.f, f = tp.noise_freq;
    for (int o = 0; o < tp.noise_octaves; ++o) {
        sum += amp * value_noise(tp, o, qx * f, qy * f, qz * f);
        amp *= tp.noise_gain;
        f *= tp.noise_lac;
    }
    return sum * tp.noise_inv_norm;
}

// fBm at world position p (noise domain shifted by tp.noise_shift).
__device__ __forceinline__ float fbm(const TraceParams& tp, float px, float py, float pz) {
    if (tp.noise_octaves <= 0) return 1.f;
    return fbm_q(tp, px + tp.noise_shift[0], py + tp.noise_shift[1], pz + tp.noise_shift[2]);
}

}  // namespace cgs
