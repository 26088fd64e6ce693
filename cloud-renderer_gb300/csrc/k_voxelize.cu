// k_voxelize.cu -- sun-view map, highlight stores, brick-binned coverage splat
// and the mip pyramid.  Compiled with -fmad=false: every FP32 operation that
// decides an index (sun-view depth keys, highlight voxel indices) is written
// with explicitly rounded intrinsics in the same order as the CPU oracle, so
// winners, indices and integer coverage match it bit for bit.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "cg_internal.h"

namespace {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

__device__ __forceinline__ long long floor_div(long long a, long long b) {
    long long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

// Voxels whose centre (2i+1)*2^19 lies in [q-rq, q+rq], clamped to [0, D-1].
__device__ __forceinline__ bool axis_range(int q, int rq, int D, int& lo, int& hi) {
    long long l = floor_div((long long)q - rq - CG_HALF_Q20 + CG_Q20 - 1, CG_Q20);
    long long h = floor_div((long long)q + rq - CG_HALF_Q20, CG_Q20);
    if (l < 0) l = 0;
    if (h > D - 1) h = D - 1;
    if (l > h) return false;
    lo = (int)l;
    hi = (int)h;
    return true;
}

// ---- brick binning ---------------------------------------------------------

// Distance term along one axis from the board centre q to the nearest voxel
// centre of the voxel range [lo, hi] (Q20).
__device__ __forceinline__ long long axis_gap(int q, int lo, int hi) {
    long long c0 = (2ll * lo + 1) * CG_HALF_Q20, c1 = (2ll * hi + 1) * CG_HALF_Q20;
    long long c = q < c0 ? c0 : (q > c1 ? c1 : (long long)q);
    return (long long)q - c;
}

// Board bin walk shared by the count and fill passes: one warp per board,
// lanes over the bricks of its voxel box; a brick is kept only when its
// nearest voxel centre passes the board's ball test, so no brick without an
// inside voxel enters the bins (the per-voxel test in k_splat stays exact).
template <bool FILL>
__device__ __forceinline__ void bin_walk(const BoardsDev& b, int D, Bins& bins) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= b.n || b.culled[i]) return;
    const int4 q = b.q[i];
    const unsigned long long thr = b.thr[i];
    int xl, xh, yl, yh, zl, zh;
    if (!axis_range(q.x, q.w, D, xl, xh) || !axis_range(q.y, q.w, D, yl, yh) ||
        !axis_range(q.z, q.w, D, zl, zh))
        return;
    const int bx0 = xl / CG_BRICK, by0 = yl / CG_BRICK, bz0 = zl / CG_BRICK;
    const int nx = xh / CG_BRICK - bx0 + 1, ny = yh / CG_BRICK - by0 + 1,
              nz = zh / CG_BRICK - bz0 + 1;
    const int total = nx * ny * nz;
    for (int t = lane; t < total; t += 32) {
        const int bx = bx0 + t % nx, by = by0 + (t / nx) % ny, bz = bz0 + t / (nx * ny);
        long long gx = axis_gap(q.x, max(bx * CG_BRICK, xl), min(bx * CG_BRICK + 7, xh));
        long long gy = axis_gap(q.y, max(by * CG_BRICK, yl), min(by * CG_BRICK + 7, yh));
        long long gz = axis_gap(q.z, max(bz * CG_BRICK, zl), min(bz * CG_BRICK + 7, zh));
        unsigned long long d2 = (unsigned long long)(gx * gx) + (unsigned long long)(gy * gy) +
                                (unsigned long long)(gz * gz);
        if (d2 > thr) continue;
        const int brick = (bz * bins.nby + by) * bins.nbx + bx;
        if (FILL) {
            uint32_t slot = atomicAdd(&bins.cursor[brick], 1u);
            bins.list[slot] = (uint32_t)i;
        } else {
            atomicAdd(&bins.count[brick], 1u);
        }
    }
}

__global__ void k_bin_count(BoardsDev b, int D, Bins bins) { bin_walk<false>(b, D, bins); }
__global__ void k_bin_fill(BoardsDev b, int D, Bins bins) { bin_walk<true>(b, D, bins); }

// Exclusive scan of the brick counts in one CTA; seeds the cursors.  Each
// pass covers 1024 x 32 counts staged in shared memory: coalesced 16-byte
// loads into a padded array (one spare word per 32 counts, so that a
// thread's 32 consecutive counts fall in 32 different banks), per-thread sums,
// a block scan of the thread sums, the exclusive offsets written back in
// place, then coalesced 16-byte stores of offsets and cursors.  A running
// carry links the passes.  count, offset and cursor are 16-byte aligned.
constexpr int SCAN_PER = 32;
constexpr int SCAN_TILE = 1024 * SCAN_PER;
constexpr int SCAN_SMEM = (SCAN_TILE + SCAN_TILE / 32) * 4;

__device__ __forceinline__ int scan_slot(int e) { return e + (e >> 5); }

__global__ void __launch_bounds__(1024) k_bin_scan(Bins bins) {
    extern __shared__ uint32_t s_cnt[];
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry_s;
    const int n = bins.nbricks;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry_s = 0;
    for (int base = 0; base < n; base += SCAN_TILE) {
        const int m = min(SCAN_TILE, n - base);
#pragma unroll
        for (int j = 0; j < SCAN_TILE / 4096; ++j) {
            const int e = 4 * tid + 4096 * j;
            uint4 q = make_uint4(0u, 0u, 0u, 0u);
            if (e + 3 < m) {
                q = *reinterpret_cast<const uint4*>(bins.count + base + e);
            } else {
                if (e < m) q.x = bins.count[base + e];
                if (e + 1 < m) q.y = bins.count[base + e + 1];
                if (e + 2 < m) q.z = bins.count[base + e + 2];
            }
            const int sl = scan_slot(e);
            s_cnt[sl] = q.x;
            s_cnt[sl + 1] = q.y;
            s_cnt[sl + 2] = q.z;
            s_cnt[sl + 3] = q.w;
        }
        __syncthreads();
        uint32_t* mine = s_cnt + tid * (SCAN_PER + 1);
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) s += mine[k];
        uint32_t x = s;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sums[lane], z = w;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            warp_sums[lane] = z - w;
        }
        __syncthreads();
        const uint32_t carry = carry_s;
        uint32_t run = carry + warp_sums[wid] + x - s;
#pragma unroll
        for (int k = 0; k < SCAN_PER; ++k) {
            const uint32_t c = mine[k];
            mine[k] = run;
            run += c;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SCAN_TILE / 4096; ++j) {
            const int e = 4 * tid + 4096 * j;
            if (e >= m) continue;
            const int sl = scan_slot(e);
            const uint4 q = make_uint4(s_cnt[sl], s_cnt[sl + 1], s_cnt[sl + 2], s_cnt[sl + 3]);
            if (e + 3 < m) {
                *reinterpret_cast<uint4*>(bins.offset + base + e) = q;
                *reinterpret_cast<uint4*>(bins.cursor + base + e) = q;
            } else {
                const uint32_t v[4] = {q.x, q.y, q.z, q.w};
                for (int k = 0; e + k < m; ++k) {
                    bins.offset[base + e + k] = v[k];
                    bins.cursor[base + e + k] = v[k];
                }
            }
        }
        if (tid == 1023) carry_s = carry + warp_sums[wid] + x;
        __syncthreads();
    }
    if (tid == 0) bins.offset[n] = carry_s;
}

// ---- sun-view nearest-surface map (first_voxelize.glsl:39-64) --------------

__device__ __forceinline__ float dot3(const float a[3], float x, float y, float z) {
    return fadd(fadd(fmul(a[0], x), fmul(a[1], y)), fmul(a[2], z));
}

// Board centre in sun view space: lookAt rows s, u, -f plus translation.
__device__ __forceinline__ float3 sun_view_of(const SunFrame& fr, float4 c) {
    float nf[3] = {-fr.fwd[0], -fr.fwd[1], -fr.fwd[2]};
    return make_float3(fadd(dot3(fr.right, c.x, c.y, c.z), fr.t[0]),
                       fadd(dot3(fr.up, c.x, c.y, c.z), fr.t[1]),
                       fadd(dot3(nf, c.x, c.y, c.z), fr.t[2]));
}

__device__ __forceinline__ float texel_coord(float lo, float hi, int i, int n) {
    float a = fadd(__int2float_rn(i), 0.5f);
    float b = fdiv(a, __int2float_rn(n));
    return fadd(lo, fmul(b, fsub(hi, lo)));
}

// Spherical profile, discard below 0.01, surface point pushed toward the sun,
// depth from the near-plane point (first_voxelize.glsl:43-63).
__device__ __forceinline__ bool sun_fragment(float xv, float yv, float3 cv, float r,
                                             float near_z, float& zs, float& depth) {
    float dx = fsub(xv, cv.x);
    float dy = fsub(yv, cv.y);
    float d2 = fadd(fmul(dx, dx), fmul(dy, dy));
    float dist = fsqrt(d2);
    float q = fdiv(dist, r);
    float t = fsub(1.0f, fmul(q, q));
    float prof = fsqrt(t > 0.0f ? t : 0.0f);
    if (!(prof >= 0.01f)) return false;
    zs = fadd(cv.z, fmul(r, prof));
    float dz = fadd(zs, near_z);
    float dep2 = fadd(fadd(fmul(xv, xv), fmul(yv, yv)), fmul(dz, dz));
    depth = fsqrt(dep2);
    return true;
}

__device__ __forceinline__ void texel_range(float lo, float hi, float c, float r, int n,
                                            int& a, int& b) {
    float span = hi - lo;
    float l = (c - r - lo) / span * (float)n - 0.5f;
    float h = (c + r - lo) / span * (float)n - 0.5f;
    // conservative: one texel of margin each side; NaN/huge values clamp
    float fa = floorf(l) - 1.0f, fb = ceilf(h) + 1.0f;
    fa = fmaxf(fa, 0.0f);
    fb = fminf(fb, (float)(n - 1));
    if (!(fa <= fb)) { a = 1; b = 0; return; }
    a = (int)fa;
    b = (int)fb;
}

// One CTA per board.  The texel-centre coordinates of the board's box are
// tabulated once (one division per column and per row instead of two per
// texel); each warp then takes rows and sweeps, with consecutive lanes on
// consecutive texels, only the columns of the row's chord through the disc
// (d^2 <= 1.0001 r^2, widened by one texel each side; the per-texel test
// below still applies, so the chord only drops texels it would reject).
constexpr int SUN_TAB = 1024;

__device__ __forceinline__ float sun_x(const SunFrame& fr, const float* tab, bool tabbed, int ia,
                                       int ti) {
    return tabbed ? tab[ti - ia] : texel_coord(fr.lo, fr.hi, ti, fr.W);
}

__global__ void __launch_bounds__(256) k_sunmap(BoardsDev b, SunFrame fr,
                                                unsigned long long* keys) {
    __shared__ float s_x[SUN_TAB], s_y[SUN_TAB];
    const int i = blockIdx.x;
    if (i >= b.n) return;
    float4 c = b.cwr[i];
    float3 cv = sun_view_of(fr, c);
    float r = c.w;
    int ia, ib, ja, jb;
    texel_range(fr.lo, fr.hi, cv.x, r, fr.W, ia, ib);
    texel_range(fr.lo, fr.hi, cv.y, r, fr.H, ja, jb);
    if (ia > ib || ja > jb) return;
    const int nx = ib - ia + 1, ny = jb - ja + 1;
    const bool tabbed = nx <= SUN_TAB && ny <= SUN_TAB;
    if (tabbed) {
        for (int t = threadIdx.x; t < nx; t += blockDim.x)
            s_x[t] = texel_coord(fr.lo, fr.hi, ia + t, fr.W);
        for (int t = threadIdx.x; t < ny; t += blockDim.x)
            s_y[t] = texel_coord(fr.lo, fr.hi, ja + t, fr.H);
        __syncthreads();
    }
    const float r2 = 1.0001f * (r * r);
    // the surface offset dz = (cv.z + r * prof) + near_z over prof in [0, 1]
    // spans [dz_lo, dz_hi] (rounded steps are monotone): its smallest square
    float dz2_min = 0.0f;
    {
        const float dz_lo = fadd(cv.z, fr.near_z), dz_hi = fadd(fadd(cv.z, r), fr.near_z);
        if (dz_lo > 0.0f) dz2_min = fmul(dz_lo, dz_lo);
        else if (dz_hi < 0.0f) dz2_min = fmul(dz_hi, dz_hi);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const float span = fr.hi - fr.lo;
    for (int row = warp; row < ny; row += nwarps) {
        const int tj = ja + row;
        const float yv = tabbed ? s_y[row] : texel_coord(fr.lo, fr.hi, tj, fr.H);
        const float ey = yv - cv.y;
        const float rem = r2 - ey * ey;
        if (!(rem >= 0.f)) continue;  // the whole row is outside the disc
        // the chord's texels, one texel of margin each side, within the box
        const float w = sqrtf(rem);
        int ca = (int)fmaxf(floorf((cv.x - w - fr.lo) / span * (float)fr.W - 0.5f) - 1.0f,
                            (float)ia);
        int cb = (int)fminf(ceilf((cv.x + w - fr.lo) / span * (float)fr.W - 0.5f) + 1.0f,
                            (float)ib);
        unsigned long long* krow = keys + (size_t)tj * fr.W;
        for (int ti = ca + lane; ti <= cb; ti += 32) {
            const float xv = sun_x(fr, s_x, tabbed, ia, ti);
            // texels well outside the disc (d^2 > 1.0001 r^2, where the exact
            // profile test cannot pass) skip the square roots and the division
            {
                const float ex = xv - cv.x;
                if (ex * ex + ey * ey > r2) continue;
            }
            unsigned long long* k = krow + ti;
            // values only decrease, so a stale read can only make the tests
            // below pass (never skip a winner)
            const unsigned long long cur = *(volatile unsigned long long*)k;
            // a certain loser skips the square roots and the division: this
            // board's depth here is at least sqrt(xy2 + dz_min^2) (every step
            // of the depth is monotone in |dz|), and a current depth whose
            // square is below that by 2^-20 relative is strictly smaller as a
            // float; an empty texel (all ones, a NaN) never skips
            {
                const float xy2 = fadd(fmul(xv, xv), fmul(yv, yv));
                const float cd = __uint_as_float((unsigned)(cur >> 32));
                if (cd * cd < fadd(xy2, dz2_min) * (1.0f - 0x1p-20f)) continue;
            }
            float zs, depth;
            if (!sun_fragment(xv, yv, cv, r, fr.near_z, zs, depth)) continue;
            unsigned long long key =
                ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned)i;
            if (key < cur) atomicMin(k, key);
        }
    }
}

// ---- highlight stores (second_voxelize.glsl:34-51) -------------------------

struct HiParams {
    float wmin[3], range[3];
    float fD, offset;
    int D;
    int nb;            // bricks per axis
    uint8_t* hl;       // per-brick highlight flags (NULL: none)
};

__device__ __forceinline__ bool voxel_index(const HiParams& hp, float x, float y, float z,
                                            int& o, int& brick) {
    float c[3] = {x, y, z};
    int id[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float t = fdiv(fsub(c[a], hp.wmin[a]), hp.range[a]);
        float v = fmul(hp.fD, t);
        if (!(v > -1.0f && v < hp.fD)) return false;
        id[a] = __float2int_rz(v);  // ivec3(): truncation toward zero
    }
    o = (id[2] * hp.D + id[1]) * hp.D + id[0];
    brick = ((id[2] / CG_BRICK) * hp.nb + id[1] / CG_BRICK) * hp.nb + id[0] / CG_BRICK;
    return true;
}

// One highlight store: the voxel's mask byte and, when flags are kept, its
// brick's flag.
__device__ __forceinline__ void mark(const HiParams& hp, uint8_t* mask, int vi, int brick) {
    if (!CG_IN_BOUNDS(vi, (size_t)hp.D * hp.D * hp.D)) return;
    mask[vi] = 1;
    if (hp.hl && CG_IN_BOUNDS(brick, (size_t)hp.nb * hp.nb * hp.nb)) hp.hl[brick] = 1;
}

__global__ void k_highlight(BoardsDev b, SunFrame fr, const unsigned long long* keys,
                            float4* posmap, HiParams hp, uint8_t* mask) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x;
    const int tj = blockIdx.y * blockDim.y + threadIdx.y;
    if (ti >= fr.W || tj >= fr.H) return;
    const size_t idx = (size_t)tj * fr.W + ti;
    unsigned long long key = keys[idx];
    if (key == CG_KEY_EMPTY) {
        posmap[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    int bi = (int)(key & 0xFFFFFFFFull);
    float4 c = b.cwr[bi];
    float3 cv = sun_view_of(fr, c);
    float xv = texel_coord(fr.lo, fr.hi, ti, fr.W);
    float yv = texel_coord(fr.lo, fr.hi, tj, fr.H);
    float zs = 0.f, depth = 0.f;
    sun_fragment(xv, yv, cv, c.w, fr.near_z, zs, depth);
    float p[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        p[a] = fadd(fadd(fadd(fmul(xv, fr.right[a]), fmul(yv, fr.up[a])), fmul(zs, -fr.fwd[a])),
                    fr.eye[a]);
    posmap[idx] = make_float4(p[0], p[1], p[2], 1.0f);
    const float o = hp.offset;
    int vi, bk;
    if (voxel_index(hp, p[0], p[1], p[2], vi, bk)) mark(hp, mask, vi, bk);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float x = (k & 4) ? fsub(p[0], o) : fadd(p[0], o);
        float y = (k & 2) ? fsub(p[1], o) : fadd(p[1], o);
        float z = (k & 1) ? fsub(p[2], o) : fadd(p[2], o);
        if (voxel_index(hp, x, y, z, vi, bk)) mark(hp, mask, vi, bk);
    }
}

// ---- coverage splat + level 0 + fused mips ---------------------------------

__device__ __forceinline__ uint32_t pack_bf16_fp16(float r, float g) {
    __nv_bfloat16 rb = __float2bfloat16_rn(r);
    __half gh = __float2half_rn(g);
    return (uint32_t)__bfloat16_as_ushort(rb) | ((uint32_t)__half_as_ushort(gh) << 16);
}

__device__ __forceinline__ float4 unpack_bf16_fp16(uint32_t v) {
    float r = __bfloat162float(__ushort_as_bfloat16((unsigned short)(v & 0xFFFFu)));
    float g = __half2float(__ushort_as_half((unsigned short)(v >> 16)));
    return make_float4(r, g, 0.f, 0.f);
}

__device__ __forceinline__ void store_voxel(const VolDesc& vd, void* pyr, int l, int x, int y,
                                            int z, float4 v) {
    const int N = vd.dims[l];
    size_t idx = (size_t)vd.offs[l] + ((size_t)z * N + y) * N + x;
    if (!CG_IN_BOUNDS(idx, vd.nvox)) return;
    __half2 h;
    if (vd.fmt == 0) {
        reinterpret_cast<float4*>(pyr)[idx] = v;
        h = __floats2half2_rn(v.x, v.y);
    } else {
        const uint32_t w = pack_bf16_fp16(v.x, v.y);
        reinterpret_cast<uint32_t*>(pyr)[idx] = w;
        h = __halves2half2(__float2half_rn(__uint_as_float(w << 16)),
                           __ushort_as_half((unsigned short)(w >> 16)));
    }
    // the half2 texture copy holds exactly what the level stores (the same
    // conversion as the copy pass of k_textures.cu)
    if (vd.surf[l]) surf3Dwrite(*reinterpret_cast<uint32_t*>(&h), vd.surf[l], x * 4, y, z);
}

__device__ __forceinline__ float4 load_voxel(const VolDesc& vd, const void* pyr, int l, int x,
                                             int y, int z) {
    const int N = vd.dims[l];
    size_t idx = (size_t)vd.offs[l] + ((size_t)z * N + y) * N + x;
    if (vd.fmt == 0) return reinterpret_cast<const float4*>(pyr)[idx];
    return unpack_bf16_fp16(reinterpret_cast<const uint32_t*>(pyr)[idx]);
}

__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
// 2x2x2 box mean in the oracle's order: ((c000+c100)+(c010+c110)) + ((c001+c101)+(c011+c111))
__device__ __forceinline__ float4 box8(float4 c000, float4 c100, float4 c010, float4 c110,
                                       float4 c001, float4 c101, float4 c011, float4 c111) {
    float4 s = f4add(f4add(f4add(c000, c100), f4add(c010, c110)),
                     f4add(f4add(c001, c101), f4add(c011, c111)));
    return make_float4(s.x * 0.125f, s.y * 0.125f, s.z * 0.125f, s.w * 0.125f);
}

// One CTA per 8^3 brick, 64 threads, one (x, y) column of eight voxels per
// thread (each staged board is tested against all eight with one set of
// shared-memory reads and one dx^2 + dy^2; a column that misses the ball
// skips its eight tests).
// Boards of the brick's bin are staged through shared memory; each voxel
// tests its centre against each board's ball on the Q20 grid (int64 squared
// distance) and sums count and Q16.16 density.
// COV = false (voxelize): level 0 is assembled in registers, the next
// `fused_levels` mip levels are reduced in shared memory, raw occupancy is
// flagged.  COV = true: only the integer coverage (count, dq) is written
// (the coverage readback and the active-voxel statistic compute it on demand).
template <bool COV>
__global__ void __launch_bounds__(64) k_splat(BoardsDev b, Bins bins, const uint8_t* mask,
                                               VolDesc vd, void* pyr, uint32_t* count,
                                               uint32_t* dqout, int fused_levels,
                                               OccRaw occ_raw) {
    // the staged boards and, once every thread has left the board loop, the
    // brick's level-0 tile share one buffer (more resident bricks per SM)
    static_assert(CG_SPLAT_CHUNK * 28 <= CG_BRICK * CG_BRICK * CG_BRICK * 16,
                  "board chunk larger than the tile it shares memory with");
    __shared__ __align__(16) uint8_t s_buf[CG_BRICK * CG_BRICK * CG_BRICK * 16];
    int4* sq = reinterpret_cast<int4*>(s_buf);
    unsigned long long* sthr = reinterpret_cast<unsigned long long*>(s_buf + CG_SPLAT_CHUNK * 16);
    uint32_t* sdq = reinterpret_cast<uint32_t*>(s_buf + CG_SPLAT_CHUNK * 24);
    float4* tile = reinterpret_cast<float4*>(s_buf);
    __shared__ unsigned s_cells;  // raw occupancy of the brick's eight 4^3 cells
    __shared__ float4 tile1[64];
    __shared__ float4 tile2[8];

    const int brick = blockIdx.x;
    const int bx = brick % bins.nbx;
    const int by = (brick / bins.nbx) % bins.nby;
    const int bz = brick / (bins.nbx * bins.nby);
    const int tid = threadIdx.x;
    // voxel j of the thread: (lx, ly, j), tile index tid + 64 j
    const int lx = tid & 7, ly = (tid >> 3) & 7, lz = 0;
    const int D = vd.D;
    const int x = bx * CG_BRICK + lx, y = by * CG_BRICK + ly;
    const int z0 = bz * CG_BRICK + lz;
    const bool inxy = x < D && y < D;
    const int vx = (2 * x + 1) * (int)CG_HALF_Q20;
    const int vy = (2 * y + 1) * (int)CG_HALF_Q20;
    const int vz0 = (2 * z0 + 1) * (int)CG_HALF_Q20;
    constexpr int DZ = 2 * (int)CG_HALF_Q20;  // one voxel along z

    const uint32_t beg = bins.offset[brick];
    const uint32_t n = bins.offset[brick + 1] - beg;
    uint32_t cnt[8] = {}, dsum[8] = {};
    const int w = tid >> 5;
    for (uint32_t base = 0; base < n; base += CG_SPLAT_CHUNK) {
        const uint32_t m = min((uint32_t)CG_SPLAT_CHUNK, n - base);
        __syncthreads();
        for (uint32_t t = tid; t < m; t += blockDim.x) {
            uint32_t bi = bins.list[beg + base + t];
            sq[t] = b.q[bi];
            sthr[t] = b.thr[bi];
            sdq[t] = b.dq[bi];
        }
        __syncthreads();
        for (uint32_t k = 0; k < m; ++k) {
            const int4 q = sq[k];
            const unsigned long long thr = sthr[k];
            const uint32_t dq = sdq[k];
            const int dx = vx - q.x, dy = vy - q.y;
            const unsigned long long dxy = (unsigned long long)((long long)dx * dx) +
                                           (unsigned long long)((long long)dy * dy);
            if (dxy > thr) continue;  // the column misses the ball
            int dz = vz0 - q.z;
#pragma unroll
            for (int j = 0; j < 8; ++j, dz += DZ) {
                const unsigned long long d = dxy + (unsigned long long)((long long)dz * dz);
                if (d <= thr) {
                    cnt[j] += 1u;
                    dsum[j] += dq;
                }
            }
        }
    }
    if (COV) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int z = z0 + j;
            if (!(inxy && z < D)) continue;
            const size_t i = ((size_t)z * D + y) * D + x;
            count[i] = cnt[j];
            dqout[i] = dsum[j];
        }
        return;
    }
    // Raw occupancy (4^3 cells, every level): the brick's eight level-0 cells
    // from its voxels, and at level l >= 1 the one cell holding the brick
    // (level-l cell = brick >> (l - 1)).  Idempotent byte stores into grids
    // cleared before the launch; k_occ_dilate builds the brick grids.
    if (tid == 0) s_cells = 0u;
    // the brick's highlight bits, then one block decision (which is also the
    // barrier after the board loop: the tile may be written): a brick without
    // boards or highlights whose voxels are still zero from an earlier
    // voxelize writes nothing
    // (with per-brick flags, a brick no highlight store touched reads none of
    // its 512 mask bytes)
    const bool hl = bins.hl == nullptr || bins.hl[brick] != 0;
    unsigned mkb = 0u;
    if (hl) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int z = z0 + j;
            if (inxy && z < D && mask[((size_t)z * D + y) * D + x]) mkb |= 1u << j;
        }
    }
    const bool keep = n > 0u || (hl && __syncthreads_or(mkb != 0u));
    if (!keep && !bins.dirty[brick]) return;
    __syncthreads();  // every thread has read the flag
    if (tid == 0) bins.dirty[brick] = keep ? 1 : 0;
    {
        // the warp's voxels lie in cell y = w & 1; voxel j in cell z = j >> 2;
        // lanes 0-3 of each row of 8 in x cell 0, lanes 4-7 in x cell 1
        const int cy = 2 * (w & 1);
        unsigned bits = 0u;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int z = z0 + j;
            const bool in = inxy && z < D;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (in) {
                const bool mk = (mkb >> j) & 1u;
                v.x = __uint2float_rn(dsum[j]) * (1.0f / 65536.0f);
                v.y = mk ? 1.0f : 0.0f;
                v.z = __uint2float_rn(cnt[j]);
                v.w = (cnt[j] > 0u || mk) ? 1.0f : 0.0f;
                store_voxel(vd, pyr, 0, x, y, z, v);
            }
            if (fused_levels > 0) tile[tid + 64 * j] = v;  // voxel (lx, ly, j)
            // density v.x > 0 exactly when dsum > 0
            const unsigned bal = __ballot_sync(0xffffffffu, in && dsum[j] > 0u);
            const int cz = 4 * (j >> 2);
            if (bal & 0x0F0F0F0Fu) bits |= 1u << (cy + cz);
            if (bal & 0xF0F0F0F0u) bits |= 1u << (cy + cz + 1);
        }
        if ((tid & 31) == 0 && bits) atomicOr(&s_cells, bits);
    }
    __syncthreads();
    const unsigned cells = s_cells;
    if (cells && tid < 8 + vd.L - 1) {
        int l, cx, cy, cz;
        bool set;
        if (tid < 8) {
            l = 0;
            set = (cells >> tid) & 1u;
            cx = 2 * bx + (tid & 1);
            cy = 2 * by + ((tid >> 1) & 1);
            cz = 2 * bz + (tid >> 2);
        } else {
            l = tid - 7;
            set = true;
            cx = bx >> (l - 1);
            cy = by >> (l - 1);
            cz = bz >> (l - 1);
        }
        const int nb = occ_raw.nb[l];
        if (set) {
            cx = min(cx, nb - 1);
            cy = min(cy, nb - 1);
            cz = min(cz, nb - 1);
            uint8_t* p = occ_raw.raw + occ_raw.off[l] + ((size_t)cz * nb + cy) * nb + cx;
            if (!*(volatile uint8_t*)p) *p = 1;
        }
    }
    if (fused_levels <= 0) return;
    // level 1: 4^3 parents
    if (tid < 64) {
        int px = tid & 3, py = (tid >> 2) & 3, pz = tid >> 4;
#define T8(a, b2, c) tile[((2 * pz + (c)) * 8 + (2 * py + (b2))) * 8 + (2 * px + (a))]
        float4 m1 = box8(T8(0, 0, 0), T8(1, 0, 0), T8(0, 1, 0), T8(1, 1, 0), T8(0, 0, 1),
                         T8(1, 0, 1), T8(0, 1, 1), T8(1, 1, 1));
#undef T8
        int gx = bx * 4 + px, gy = by * 4 + py, gz = bz * 4 + pz;
        if (gx < vd.dims[1] && gy < vd.dims[1] && gz < vd.dims[1])
            store_voxel(vd, pyr, 1, gx, gy, gz, m1);
        tile1[tid] = m1;
    }
    __syncthreads();
    if (fused_levels < 2) return;
    if (tid < 8) {
        int px = tid & 1, py = (tid >> 1) & 1, pz = tid >> 2;
#define T4(a, b2, c) tile1[((2 * pz + (c)) * 4 + (2 * py + (b2))) * 4 + (2 * px + (a))]
        float4 m2 = box8(T4(0, 0, 0), T4(1, 0, 0), T4(0, 1, 0), T4(1, 1, 0), T4(0, 0, 1),
                         T4(1, 0, 1), T4(0, 1, 1), T4(1, 1, 1));
#undef T4
        int gx = bx * 2 + px, gy = by * 2 + py, gz = bz * 2 + pz;
        if (gx < vd.dims[2] && gy < vd.dims[2] && gz < vd.dims[2])
            store_voxel(vd, pyr, 2, gx, gy, gz, m2);
        tile2[tid] = m2;
    }
    __syncthreads();
    if (fused_levels < 3) return;
    if (tid == 0) {
        float4 m3 = box8(tile2[0], tile2[1], tile2[2], tile2[3], tile2[4], tile2[5], tile2[6],
                         tile2[7]);
        if (bx < vd.dims[3] && by < vd.dims[3] && bz < vd.dims[3])
            store_voxel(vd, pyr, 3, bx, by, bz, m3);
    }
}

// Dilated occupancy: occ[l][c] = 1 when a raw 4^3 cell of level l inside
// brick c (B = 1 << occ_shift texels) or one of its 26 neighbours is set; one
// thread per brick of every level.  The occupied level-0 bricks also grow the
// level-0 box (box[0..2] = D - lo, box[3..5] = hi, atomic maxima from zero).
__global__ void __launch_bounds__(256) k_occ_dilate(VolDesc vd, OccRaw raw, uint8_t* occ,
                                                    int total, int* box) {
    __shared__ unsigned s_box[8][6];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned m[6] = {0u, 0u, 0u, 0u, 0u, 0u};  // this brick's box terms (0 = none)
    if (i < total) {
        int l = 0;
        while (l + 1 < vd.L && i >= vd.occ_off[l + 1]) ++l;
        const int nb = vd.occ_nb[l], r = i - vd.occ_off[l];
        const int cx = r % nb, cy = (r / nb) % nb, cz = r / (nb * nb);
        const int k = vd.occ_shift - 2;  // raw cells per brick edge: 1 << k
        const int rn = raw.nb[l];
        const uint8_t* g = raw.raw + raw.off[l];
        const int x0 = max((cx - 1) << k, 0), x1 = min((cx + 2) << k, rn);
        const int y0 = max((cy - 1) << k, 0), y1 = min((cy + 2) << k, rn);
        const int z0 = max((cz - 1) << k, 0), z1 = min((cz + 2) << k, rn);
        uint8_t any = 0;
        for (int z = z0; z < z1 && !any; ++z)
            for (int y = y0; y < y1 && !any; ++y)
                for (int x = x0; x < x1; ++x) any |= g[((size_t)z * rn + y) * rn + x];
        occ[i] = any ? 1 : 0;
        if (any && l == 0) {
            const int B = 1 << vd.occ_shift, D = vd.D;
            const int c[3] = {cx, cy, cz};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                m[a] = (unsigned)(D - c[a] * B);
                m[3 + a] = (unsigned)min(D, (c[a] + 1) * B);
            }
        }
    }
    // the occupied level-0 box: block maxima (warp reductions, then warp 0),
    // one atomic per value per block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 6; ++a) m[a] = __reduce_max_sync(0xffffffffu, m[a]);
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < 6; ++a) s_box[w][a] = m[a];
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            const unsigned v = __reduce_max_sync(0xffffffffu, lane < nw ? s_box[lane][a] : 0u);
            if (lane == 0 && v > 0u) atomicMax(box + a, (int)v);
        }
    }
}

// Parent (x, y, z) of level l + 1 as the mean of its 2x2x2 children at level
// l (clamped at odd edges).
__device__ __forceinline__ void mip_parent(const VolDesc& vd, void* pyr, int l, int x, int y,
                                           int z) {
    const int Nc = vd.dims[l];
    int cx0 = min(2 * x, Nc - 1), cx1 = min(2 * x + 1, Nc - 1);
    int cy0 = min(2 * y, Nc - 1), cy1 = min(2 * y + 1, Nc - 1);
    int cz0 = min(2 * z, Nc - 1), cz1 = min(2 * z + 1, Nc - 1);
    float4 m = box8(load_voxel(vd, pyr, l, cx0, cy0, cz0), load_voxel(vd, pyr, l, cx1, cy0, cz0),
                    load_voxel(vd, pyr, l, cx0, cy1, cz0), load_voxel(vd, pyr, l, cx1, cy1, cz0),
                    load_voxel(vd, pyr, l, cx0, cy0, cz1), load_voxel(vd, pyr, l, cx1, cy0, cz1),
                    load_voxel(vd, pyr, l, cx0, cy1, cz1), load_voxel(vd, pyr, l, cx1, cy1, cz1));
    store_voxel(vd, pyr, l + 1, x, y, z, m);
}

// Generic 2x2x2 reduction from level l to l+1 (one thread per parent).
__global__ void k_mip_level(VolDesc vd, void* pyr, int l) {
    const int Np = vd.dims[l + 1];
    const long long total = (long long)Np * Np * Np;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    mip_parent(vd, pyr, l, (int)(i % Np), (int)((i / Np) % Np), (int)(i / ((long long)Np * Np)));
}

// The small levels l0+1 .. L-1 in one CTA, level after level (a block
// barrier makes each level's stores visible to the next level's loads).
__global__ void __launch_bounds__(1024) k_mip_tail(VolDesc vd, void* pyr, int l0) {
    for (int l = l0; l + 1 < vd.L; ++l) {
        const int Np = vd.dims[l + 1];
        const int total = Np * Np * Np;
        for (int i = threadIdx.x; i < total; i += blockDim.x)
            mip_parent(vd, pyr, l, i % Np, (i / Np) % Np, i / (Np * Np));
        __syncthreads();
    }
}

__global__ void k_count_active(const uint32_t* count, const uint8_t* mask, size_t n,
                               unsigned long long* out) {
    unsigned long long local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        local += (count[i] > 0u || mask[i]) ? 1ull : 0ull;
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}

}  // namespace

cudaError_t launch_bin_count(const BoardsDev& b, int D, Bins bins, cudaStream_t st) {
    if (b.n == 0) return cudaSuccess;
    k_bin_count<<<(b.n + 3) / 4, 128, 0, st>>>(b, D, bins);  // one warp per board
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(Bins bins, cudaStream_t st) {
    // the shared-memory attribute is set once per device (atomics keep
    // concurrent host threads well-defined)
    static std::atomic<bool> configured[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!configured[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(k_bin_scan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 SCAN_SMEM);
        if (e != cudaSuccess) return e;
        configured[dev].store(true, std::memory_order_release);
    }
    k_bin_scan<<<1, 1024, SCAN_SMEM, st>>>(bins);
    return cudaGetLastError();
}

cudaError_t launch_bin_fill(const BoardsDev& b, int D, Bins bins, cudaStream_t st) {
    if (b.n == 0) return cudaSuccess;
    k_bin_fill<<<(b.n + 3) / 4, 128, 0, st>>>(b, D, bins);
    return cudaGetLastError();
}

cudaError_t launch_sunmap(const BoardsDev& b, const SunFrame& fr, uint64_t* keys,
                          cudaStream_t st) {
    if (b.n == 0) return cudaSuccess;
    k_sunmap<<<b.n, 256, 0, st>>>(b, fr, reinterpret_cast<unsigned long long*>(keys));
    return cudaGetLastError();
}

cudaError_t launch_highlight(const BoardsDev& b, const SunFrame& fr, const uint64_t* keys,
                             float4* posmap, int D, const float wmin[3],
                             const float range[3], float offset, uint8_t* mask,
                             uint8_t* hl_brick, cudaStream_t st) {
    HiParams hp;
    hp.nb = (D + CG_BRICK - 1) / CG_BRICK;
    hp.hl = hl_brick;
    for (int a = 0; a < 3; ++a) {
        hp.wmin[a] = wmin[a];
        hp.range[a] = range[a];
    }
    hp.fD = (float)D;
    hp.offset = offset;
    hp.D = D;
    dim3 blk(32, 8);
    dim3 grd((fr.W + 31) / 32, (fr.H + 7) / 8);
    k_highlight<<<grd, blk, 0, st>>>(b, fr, reinterpret_cast<const unsigned long long*>(keys),
                                     posmap, hp, mask);
    return cudaGetLastError();
}

cudaError_t launch_splat(const BoardsDev& b, Bins bins, const uint8_t* mask, VolDesc vd,
                         void* pyr, uint32_t* count, uint32_t* dq, int fused_levels,
                         OccRaw occ, bool coverage_only, cudaStream_t st) {
    if (coverage_only)
        k_splat<true><<<bins.nbricks, 64, 0, st>>>(b, bins, mask, vd, pyr, count, dq,
                                                    fused_levels, occ);
    else
        k_splat<false><<<bins.nbricks, 64, 0, st>>>(b, bins, mask, vd, pyr, count, dq,
                                                     fused_levels, occ);
    return cudaGetLastError();
}

cudaError_t launch_occ_dilate(VolDesc vd, OccRaw raw, uint8_t* occ, int total, cudaStream_t st) {
    k_occ_dilate<<<(total + 255) / 256, 256, 0, st>>>(vd, raw, occ, total,
                                                      const_cast<int*>(vd.occ_box));
    return cudaGetLastError();
}

cudaError_t launch_mip_level(VolDesc vd, void* pyr, int l, cudaStream_t st) {
    long long np = (long long)vd.dims[l + 1];
    long long total = np * np * np;
    int blocks = (int)((total + 255) / 256);
    k_mip_level<<<blocks, 256, 0, st>>>(vd, pyr, l);
    return cudaGetLastError();
}

cudaError_t launch_mip_tail(VolDesc vd, void* pyr, int l0, cudaStream_t st) {
    k_mip_tail<<<1, 1024, 0, st>>>(vd, pyr, l0);
    return cudaGetLastError();
}

cudaError_t launch_count_active(const uint32_t* count, const uint8_t* mask, size_t n,
                                unsigned long long* out, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_count_active<<<blocks, 256, 0, st>>>(count, mask, n, out);
    return cudaGetLastError();
}

CG_OOB_TU(k_voxelize)
