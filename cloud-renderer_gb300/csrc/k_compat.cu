// k_compat.cu -- the compat render: the reference's own image formation
// (ConeTraceShader::coneTrace, ConeTraceShader.cpp:15-82) as tiled kernels.
//
// The reference draws one camera-facing quad per board (radius r, centre c;
// billboard_vert_instanced.glsl with Library::createQuad), shades every
// fragment with conetrace_frag.glsl:122-201 and blends back to front
// (SRC_ALPHA, ONE_MINUS_SRC_ALPHA, main.cpp:94-95) after sorting the boards by
// distance on the CPU (CloudVolume.cpp:65-82).  Here:
//   count  one warp per board: the quad's conservative pixel rectangle, its
//          8x8 tiles (atomic per-tile counts) and the squared eye distance;
//   scan   the per-tile counts (k_bin_scan);
//   fill   one warp per board: (distance bits << 32 | board) into each
//          tile's list;
//   tiles  one 256-thread CTA per 8x8 tile: sorts its list (bitonic, in
//          shared memory up to 4096 entries, in place in global memory
//          beyond); four threads per pixel blend a quarter of the list each
//          front to back, C += T a src, T *= 1 - a, and the quarters combine
//          in order (the over operator is associative), which equals the
//          back-to-front blend; a thread stops once its T falls below the
//          cutoff, a warp once all its threads have.
// The quad is perpendicular to the view axis f, so the fragment of pixel ray
// d (d.f = 1) is the plane point e + z d with z = (c - e).f; the quad covers
// the pixel when both plane coordinates (x, y) = ((p - c).s, (p - c).u) / r
// lie in [-1, 1].
#include <cuda_runtime.h>

#include "cg_internal.h"
#include "cg_sample.cuh"

namespace {

constexpr int CAP = 4096;      // sort keys held in shared memory per tile
constexpr int NOISE_N = 32;    // noise map edge (ConeTraceShader.cpp:12)

// One warp per board: lane 0 derives the board's tile rectangle, the lanes
// split its tiles for the per-tile count.
__global__ void k_compat_count(CompatDev P, int4* rect, float* key, uint32_t* tile_count,
                               unsigned long long* pairs) {
    const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= P.n) return;
    int4 R = make_int4(1, 1, 0, 0);
    if (lane == 0) {
        const CamDesc& cam = P.cam;
        const float4 c = P.cwr[b];
        const float dx = c.x - cam.eye[0], dy = c.y - cam.eye[1], dz = c.z - cam.eye[2];
        const float z = dx * cam.f[0] + dy * cam.f[1] + dz * cam.f[2];
        key[b] = dx * dx + dy * dy + dz * dz;
        if (z > P.near_z && z < 2500.f && c.w > 0.f) {
            // plane coordinates of the centre and the half extent at unit depth
            const float xs = (dx * cam.s[0] + dy * cam.s[1] + dz * cam.s[2]) / z;
            const float ys = (dx * cam.u[0] + dy * cam.u[1] + dz * cam.u[2]) / z;
            const float h = c.w / z;
            const float ta = cam.tanh * cam.aspect;
            // pixel i lies at ndc (2 (i + 0.5) / W - 1) ta; row j at (1 - 2 (j + 0.5) / H) tanh;
            // one pixel of margin either side, the exact test is per pixel
            float lo_x = ((xs - h) / ta + 1.f) * 0.5f * (float)cam.W - 0.5f;
            float hi_x = ((xs + h) / ta + 1.f) * 0.5f * (float)cam.W - 0.5f;
            float lo_y = (1.f - (ys + h) / cam.tanh) * 0.5f * (float)cam.H - 0.5f;
            float hi_y = (1.f - (ys - h) / cam.tanh) * 0.5f * (float)cam.H - 0.5f;
            lo_x = fmaxf(lo_x, -2.f);
            lo_y = fmaxf(lo_y, -2.f);
            hi_x = fminf(hi_x, (float)cam.W + 1.f);
            hi_y = fminf(hi_y, (float)cam.H + 1.f);
            const int i0 = max(0, (int)floorf(lo_x) - 1), i1 = min(cam.W - 1, (int)ceilf(hi_x) + 1);
            const int j0 = max(0, (int)floorf(lo_y) - 1), j1 = min(cam.H - 1, (int)ceilf(hi_y) + 1);
            if (i0 <= i1 && j0 <= j1)
                R = make_int4(i0 / CG_COMPAT_TILE, j0 / CG_COMPAT_TILE, i1 / CG_COMPAT_TILE,
                              j1 / CG_COMPAT_TILE);
        }
        rect[b] = R;
    }
    R.x = __shfl_sync(0xffffffffu, R.x, 0);
    R.y = __shfl_sync(0xffffffffu, R.y, 0);
    R.z = __shfl_sync(0xffffffffu, R.z, 0);
    R.w = __shfl_sync(0xffffffffu, R.w, 0);
    const int nx = R.z - R.x + 1, ny = R.w - R.y + 1;
    if (nx <= 0 || ny <= 0) return;
    if (lane == 0) atomicAdd(pairs, (unsigned long long)nx * (unsigned long long)ny);
    for (int t = lane; t < nx * ny; t += 32)
        atomicAdd(tile_count + (R.y + t / nx) * P.tiles_x + R.x + t % nx, 1u);
}

// One warp per board: the lanes split its tiles.
__global__ void k_compat_fill(CompatDev P, const int4* rect, const float* key, uint32_t* cursor,
                              unsigned long long* list) {
    const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= P.n) return;
    const int4 R = rect[b];
    const int nx = R.z - R.x + 1, ny = R.w - R.y + 1;
    if (nx <= 0 || ny <= 0) return;
    const unsigned long long k =
        ((unsigned long long)__float_as_uint(key[b]) << 32) | (unsigned long long)(unsigned)b;
    for (int t = lane; t < nx * ny; t += 32) {
        const uint32_t slot = atomicAdd(cursor + (R.y + t / nx) * P.tiles_x + R.x + t % nx, 1u);
        list[slot] = k;
    }
}

// Ascending sort of a[0, m) by a sorting network over the next power of two
// p >= m whose every comparator puts the smaller key at the lower index
// (bitonic merges with the first step of each merge mirrored); positions at or
// beyond m stand for +infinity, so comparators reaching them never swap and
// are skipped.  All threads of the CTA call it.
template <typename Ptr>
__device__ void sort_keys(Ptr a, int m) {
    int p = 1;
    while (p < m) p <<= 1;
    for (int k = 2; k <= p; k <<= 1) {
        const int hk = k >> 1;
        for (int i = threadIdx.x; i < p / 2; i += blockDim.x) {
            const int blk = i / hk, off = i - blk * hk;
            const int lo = blk * k + off, hi = blk * k + k - 1 - off;
            if (hi < m) {
                const unsigned long long x = a[lo], y = a[hi];
                if (y < x) {
                    a[lo] = y;
                    a[hi] = x;
                }
            }
        }
        __syncthreads();
        for (int j = hk >> 1; j >= 1; j >>= 1) {
            for (int i = threadIdx.x; i < p / 2; i += blockDim.x) {
                const int blk = i / j, off = i - blk * j;
                const int lo = blk * 2 * j + off, hi = lo + j;
                if (hi < m) {
                    const unsigned long long x = a[lo], y = a[hi];
                    if (y < x) {
                        a[lo] = y;
                        a[hi] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// texture(noiseMap, q).ga: LINEAR with REPEAT at normalised coordinates (the
// fragment program reads only the green and alpha channels of a noise cell).
__device__ __forceinline__ float2 noise_tap(const float2* __restrict__ tab, float qx, float qy,
                                            float qz) {
    const float x = qx * (float)NOISE_N - 0.5f, y = qy * (float)NOISE_N - 0.5f,
                z = qz * (float)NOISE_N - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float wx = x - fx, wy = y - fy, wz = z - fz;
    const int ix = ((int)fx % NOISE_N + NOISE_N) % NOISE_N;
    const int iy = ((int)fy % NOISE_N + NOISE_N) % NOISE_N;
    const int iz = ((int)fz % NOISE_N + NOISE_N) % NOISE_N;
    const int jx = (ix + 1) & (NOISE_N - 1), jy = (iy + 1) & (NOISE_N - 1),
              jz = (iz + 1) & (NOISE_N - 1);
    const int r00 = (iz * NOISE_N + iy) * NOISE_N, r01 = (iz * NOISE_N + jy) * NOISE_N,
              r10 = (jz * NOISE_N + iy) * NOISE_N, r11 = (jz * NOISE_N + jy) * NOISE_N;
    const float2 c000 = __ldg(tab + r00 + ix), c001 = __ldg(tab + r00 + jx);
    const float2 c010 = __ldg(tab + r01 + ix), c011 = __ldg(tab + r01 + jx);
    const float2 c100 = __ldg(tab + r10 + ix), c101 = __ldg(tab + r10 + jx);
    const float2 c110 = __ldg(tab + r11 + ix), c111 = __ldg(tab + r11 + jx);
    auto tri = [&](float a000, float a001, float a010, float a011, float a100, float a101,
                   float a110, float a111) {
        const float x00 = a000 + wx * (a001 - a000), x10 = a010 + wx * (a011 - a010);
        const float x01 = a100 + wx * (a101 - a100), x11 = a110 + wx * (a111 - a110);
        const float y0 = x00 + wy * (x10 - x00), y1 = x01 + wy * (x11 - x01);
        return y0 + wz * (y1 - y0);
    };
    return make_float2(tri(c000.x, c001.x, c010.x, c011.x, c100.x, c101.x, c110.x, c111.x),
                       tri(c000.y, c001.y, c010.y, c011.y, c100.y, c101.y, c110.y, c111.y));
}

__device__ __forceinline__ float sat(float x) { return fminf(fmaxf(x, 0.f), 1.f); }

// conetrace_frag.glsl:122-201 at plane point p (plane coordinates x, y) of the
// board (c, r); false when the fragment is discarded.
template <int FMT>
__device__ bool compat_fragment(const VolDesc& vd, const ConeSchedule& cs, const CompatDev& P,
                                float px, float py, float pz, float x, float y, float4 c,
                                float4& o) {
    const float bx = -P.cam.f[0], by = -P.cam.f[1], bz = -P.cam.f[2];  // toward the camera
    const float dx = px - c.x, dy = py - c.y, dz = pz - c.z;
    const float r = c.w;
    const float tx = (x + 1.f) * 0.5f, ty = (y + 1.f) * 0.5f;  // fragTex
    if (P.show_quad) {
        float sc = sqrtf(dx * dx + dy * dy + dz * dz) / r;
        sc = sqrtf(fmaxf(0.f, 1.f - sc * sc));
        const bool edge = tx < 0.01f || ty < 0.01f || tx > 0.99f || ty > 0.99f;
        const float v = edge ? 1.f : sc;
        o = make_float4(v, v, v, v);
        return true;
    }
    if (P.do_noise) {
        const float A = bx * bx + by * by + bz * bz;
        const float B = 2.f * (dx * bx + dy * by + dz * bz);
        const float C = (dx * dx + dy * dy + dz * dz) - r * r;
        const float disc = B * B - 4.f * A * C;
        if (disc < 0.01f) return false;
        const float sq = sqrtf(disc);
        const float tn = (-B - sq) / (2.f * A), tf = (-B + sq) / (2.f * A);
        const float wnx = px + bx * tn, wny = py + by * tn, wnz = pz + bz * tn;
        const float wfx = px + bx * tf, wfy = py + by * tf, wfz = pz + bz * tf;
        float ux = (wnx - c.x) / r, uy = (wny - c.y) / r, uz = (wnz - c.z) / r;
        float cx = wnx * P.inv_adjust, cy = wny * P.inv_adjust, cz = wnz * P.inv_adjust;
        const float ex = wfx * P.inv_adjust - cx, ey = wfy * P.inv_adjust - cy,
                    ez = wfz * P.inv_adjust - cz;
        float is = sqrtf(ex * ex + ey * ey + ez * ez) / P.step_size;
        is = fminf(is, (float)(P.max_steps - P.min_steps)) + (float)P.min_steps;
        const float lx = ex / (is - 1.f), ly = ey / (is - 1.f), lz = ez / (is - 1.f);
        const float oa = P.noise_opacity / (is - 1.f), la = 1.f / (is - 1.f);
        float ro = 0.f, rl = 0.f;
        for (int i = 0; (float)i < is; ++i) {
            float ng = 0.f, na = 0.f;  // the cell's green and alpha
            float fr = 1.f, pe = 1.f;
            for (int k = 0; k < P.octaves; ++k) {
                const float off = k < 3 ? P.off[k] : 0.f;
                const float2 t = noise_tap(P.noise, (cx + off) * fr, (cy + off) * fr,
                                           (cz + off) * fr);
                ng += pe * t.x;
                na += pe * t.y;
                fr *= P.freq_step;
                pe *= P.pers_step;
            }
            na = fabsf(na);
            const float uu = ux * ux + uy * uy + uz * uz;
            ng += uy / sqrtf(uu);
            ro += na * (1.f - uu);
            rl += sat(ng * 0.5f + 0.5f);
            cx += lx;
            cy += ly;
            cz += lz;
            ux += lx;
            uy += ly;
            uz += lz;
        }
        const float col = P.min_color + P.color_scale * rl * la;
        const float qx = tx - 0.5f, qy = ty - 0.5f;
        const float alpha = 1.f - sqrtf(qx * qx + qy * qy) * 2.f;
        o = make_float4(col, col, col, sat(ro * oa) * alpha);
    }
    if (P.do_cone) {
        float sc = sqrtf(dx * dx + dy * dy + dz * dz) / r;
        sc = sqrtf(fmaxf(0.f, 1.f - sc * sc));
        if (sc < 0.01f) return false;
        const float D = (float)vd.D;
        const float vx = D * ((px + bx * r * sc - vd.wmin[0]) / vd.range[0]);
        const float vy = D * ((py + by * r * sc - vd.wmin[1]) / vd.range[1]);
        const float vz = D * ((pz + bz * r * sc - vd.wmin[2]) / vd.range[2]);
        const float ind = cgs::sun_cone<FMT>(vd, cs, vx, vy, vz, P.sun[0], P.sun[1], P.sun[2]);
        if (P.do_noise) {
            o.x *= ind;
            o.y *= ind;
            o.z *= ind;
        } else {
            o = make_float4(ind, ind, ind, ind);
        }
    }
    return true;
}

// One 256-thread CTA per 8x8-pixel tile: the tile's list is sorted once,
// then split into SEG contiguous segments; thread (segment g, pixel p) blends
// its segment front to back into (C_g, T_g) and the segments are combined in
// order with the associative over operator, C = C_0 + T_0 (C_1 + T_1 (...)),
// T = T_0 T_1 ...  A segment stops early on its own transmittance (the
// combined image moves by at most the cutoff).
constexpr int SEG = 4;
constexpr int TILE_PX = CG_COMPAT_TILE * CG_COMPAT_TILE;  // 64

template <int FMT>
__global__ void __launch_bounds__(256) k_compat_tiles(VolDesc vd, ConeSchedule cs, CompatDev P,
                                                      const uint32_t* offset,
                                                      unsigned long long* list, float4* out) {
    __shared__ unsigned long long s_keys[CAP];
    __shared__ float4 s_c[SEG][TILE_PX];
    __shared__ float s_t[SEG][TILE_PX];
    const int tile = blockIdx.x;
    const int tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    const uint32_t beg = offset[tile];
    const int m = (int)(offset[tile + 1] - beg);
    const bool in_smem = m <= CAP;
    if (in_smem) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) s_keys[i] = list[beg + i];
        __syncthreads();
        sort_keys(s_keys, m);
    } else {
        sort_keys(list + beg, m);
    }
    const unsigned long long* keys = in_smem ? s_keys : list + beg;
    const CamDesc& cam = P.cam;
    const int pix = threadIdx.x & (TILE_PX - 1), seg = threadIdx.x / TILE_PX;
    const int pxi = tx * CG_COMPAT_TILE + (pix & (CG_COMPAT_TILE - 1));
    const int pyi = ty * CG_COMPAT_TILE + (pix / CG_COMPAT_TILE);
    const bool active = pxi < cam.W && pyi < cam.H;
    const float ndx = (2.f * ((float)pxi + 0.5f) / (float)cam.W - 1.f) * cam.tanh * cam.aspect;
    const float ndy = (1.f - 2.f * ((float)pyi + 0.5f) / (float)cam.H) * cam.tanh;
    const float dx = cam.f[0] + ndx * cam.s[0] + ndy * cam.u[0];
    const float dy = cam.f[1] + ndx * cam.s[1] + ndy * cam.u[1];
    const float dz = cam.f[2] + ndx * cam.s[2] + ndy * cam.u[2];
    float4 C = make_float4(0.f, 0.f, 0.f, 0.f);
    float T = 1.f;
    const bool drawing = P.show_quad || P.do_noise || P.do_cone;
    const int k0 = (int)((long long)m * seg / SEG), k1 = (int)((long long)m * (seg + 1) / SEG);
    const int span = (m + SEG - 1) / SEG;  // the longest segment: uniform trip count
    for (int i = 0; i < span && drawing; ++i) {
        if ((i & 7) == 0 && !__any_sync(0xffffffffu, active && T >= P.cutoff && k0 + i < k1))
            break;  // the whole warp is done (warp-uniform trip count)
        const int k = k0 + i;
        if (!active || T < P.cutoff || k >= k1) continue;
        const int b = (int)(unsigned)(keys[k] & 0xFFFFFFFFull);
        const float4 c = __ldg(P.cwr + b);
        const float ox = c.x - cam.eye[0], oy = c.y - cam.eye[1], oz = c.z - cam.eye[2];
        const float z = ox * cam.f[0] + oy * cam.f[1] + oz * cam.f[2];
        if (!(z > P.near_z && z < 2500.f && c.w > 0.f)) continue;
        const float px = cam.eye[0] + z * dx, py = cam.eye[1] + z * dy, pz = cam.eye[2] + z * dz;
        const float qx = px - c.x, qy = py - c.y, qz = pz - c.z;
        const float x = (qx * cam.s[0] + qy * cam.s[1] + qz * cam.s[2]) / c.w;
        const float y = (qx * cam.u[0] + qy * cam.u[1] + qz * cam.u[2]) / c.w;
        if (!(x >= -1.f && x <= 1.f && y >= -1.f && y <= 1.f)) continue;
        float4 o;
        if (!compat_fragment<FMT>(vd, cs, P, px, py, pz, x, y, c, o)) continue;
        const float a = sat(o.w);
        const float ta = T * a;
        C.x += ta * sat(o.x);
        C.y += ta * sat(o.y);
        C.z += ta * sat(o.z);
        C.w += ta * a;
        T *= 1.f - a;
    }
    s_c[seg][pix] = C;
    s_t[seg][pix] = T;
    __syncthreads();
    if (seg == 0 && active) {
        float4 A = s_c[SEG - 1][pix];
        float TA = s_t[SEG - 1][pix];
#pragma unroll
        for (int g = SEG - 2; g >= 0; --g) {  // segment g in front of the combined rest
            const float4 F = s_c[g][pix];
            const float TF = s_t[g][pix];
            A = make_float4(F.x + TF * A.x, F.y + TF * A.y, F.z + TF * A.z, F.w + TF * A.w);
            TA *= TF;
        }
        out[(size_t)pyi * cam.W + pxi] =
            make_float4(A.x + TA * P.clear[0], A.y + TA * P.clear[1], A.z + TA * P.clear[2],
                        A.w + TA * P.clear[3]);
    }
}

}  // namespace

cudaError_t launch_compat_count(const CompatDev& P, int4* rect, float* key, uint32_t* tile_count,
                                unsigned long long* pairs, cudaStream_t st) {
    if (P.n == 0) return cudaSuccess;
    k_compat_count<<<(P.n + 3) / 4, 128, 0, st>>>(P, rect, key, tile_count, pairs);
    return cudaGetLastError();
}

cudaError_t launch_compat_fill(const CompatDev& P, const int4* rect, const float* key,
                               uint32_t* cursor, unsigned long long* list, cudaStream_t st) {
    if (P.n == 0) return cudaSuccess;
    k_compat_fill<<<(P.n + 3) / 4, 128, 0, st>>>(P, rect, key, cursor, list);
    return cudaGetLastError();
}

cudaError_t launch_compat_tiles(const VolDesc& vd, const ConeSchedule& cs, const CompatDev& P,
                                const uint32_t* offset, unsigned long long* list, float4* out,
                                cudaStream_t st) {
    const int tiles = P.tiles_x * P.tiles_y;
    if (vd.fmt == 0)
        k_compat_tiles<0><<<tiles, 256, 0, st>>>(vd, cs, P, offset, list, out);
    else
        k_compat_tiles<1><<<tiles, 256, 0, st>>>(vd, cs, P, offset, list, out);
    return cudaGetLastError();
}

CG_OOB_TU(k_compat)
