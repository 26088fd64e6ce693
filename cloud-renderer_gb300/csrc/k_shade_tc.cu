// k_shade_tc.cu -- the surrogate's inference on the fifth-generation tensor
// cores: sun transmittance of every recorded view sample through the MLP
// (16 -> 64 -> 64 -> 64 SiLU -> 1, FP16 operands, FP32 accumulation).
//
// One CTA = 4 warps = one 128-row tile at a time (persistent over tiles).
// Per tile:
//   1. each thread gathers its sample, computes the 16 features (12 texture
//      taps), and writes the normalised FP16 row into the activation tile
//      (shared memory, 128B-swizzled K-major);
//   2. thread 0 issues layer 1 (one tcgen05.mma, M=128 N=64 K=16) into tensor
//      memory and commits it to an mbarrier;
//   3. each warp reads its 32 rows x 64 FP32 columns back (tcgen05.ld), adds
//      the bias, applies SiLU in FP16 pairs and writes the next activation
//      tile in place; layers 2 and 3 are 4 MMAs each (K = 64);
//   4. the last epilogue folds the 64 -> 1 output layer into FP32 FMAs, then
//      the softplus link, the transmittance and the sample's contribution.
// The weights (three 64-row tiles) are staged once per CTA.  Every mbarrier
// wait is bounded: on a timeout the CTA records an error, waits (bounded) for
// its MMA to drain, frees its tensor memory and returns.
#include <cuda_fp16.h>

#include "cg_deferred.cuh"
#include "cg_internal.h"
#include "cg_mlp.cuh"
#include "cg_sample.cuh"
#include "cg_tc.cuh"

namespace {

constexpr uint32_t TC_TMEM_COLS = 64;
constexpr unsigned TC_WAIT_LIMIT = 1u << 22;
// shared memory map (bytes from the 1024-aligned base)
constexpr int OFF_ACT = 0;               // 128 x 128 B activation tile
constexpr int OFF_W1 = 16384;            // 64 x 128 B (K = 16 used)
constexpr int OFF_W2 = OFF_W1 + 8192;    // 64 x 128 B
constexpr int OFF_W3 = OFF_W2 + 8192;    // 64 x 128 B
constexpr int OFF_BIAS = OFF_W3 + 8192;  // b1, b2, b3 (192 floats), w4 (64), b4
constexpr int OFF_BAR = OFF_BIAS + (4 * 64 + 4) * 4;
constexpr int SMEM_USED = OFF_BAR + 16;
constexpr int SMEM_BYTES = SMEM_USED + 1024;  // + alignment slack

constexpr uint32_t IDESC = tc::idesc_f16_f32(128, 64);

// row r's 8 chunks of one FP16 weight row (64 halves) into a swizzled tile
__device__ __forceinline__ void stage_row64(uint8_t* tile, int r, const __half* src, int chunks) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (c < chunks) v = *reinterpret_cast<const uint4*>(src + 8 * c);
        *reinterpret_cast<uint4*>(tile + tc::sw128_offset(r, c)) = v;
    }
}

// bias + SiLU of 32 accumulators -> 16 FP16 pairs
__device__ __forceinline__ void bias_silu32(const uint32_t (&acc)[32], const float* bias,
                                            uint32_t (&h)[16]) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float a = __uint_as_float(acc[2 * j]) + bias[2 * j];
        const float b = __uint_as_float(acc[2 * j + 1]) + bias[2 * j + 1];
        h[j] = mlp::silu_h2(mlp::pack_h2(a, b));
    }
}

// Slot of flat row i: the chunk's first region, walked forward inside its
// march CTA's group of 8 regions (padding rows past the group's samples are
// not valid).
__device__ __forceinline__ bool locate(const SampleBuf& sb, unsigned i, unsigned total,
                                       size_t& idx) {
    if (i >= total) return false;
    unsigned r = sb.chunk_region[i >> 5];
    const unsigned last = r | 7u;
    unsigned o = sb.offset[r], e = o + sb.count[r];
    while (i >= e && r < last) {
        ++r;
        o = sb.offset[r];
        e = o + sb.count[r];
    }
    if (i >= e) return false;
    idx = (size_t)r * sb.capacity + (i - o);
    return true;
}

template <int FMT>
__global__ void __launch_bounds__(128, 4) k_shade_mlp_tc(VolDesc vd, TraceParams tp,
                                                         ConeSchedule cone, MlpDev m,
                                                         SampleBuf sb,
                                                         unsigned long long* status) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_addr(smem_raw);
    uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* act = base + OFF_ACT;
    float* sBias = reinterpret_cast<float*>(base + OFF_BIAS);  // [0,192) b1..b3, [192,256) w4
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + OFF_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + OFF_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // ---- stage weights (FP16 image: W1 [64][16], W2/W3 [64][64], W4 row 0)
    for (int r = tid; r < 64; r += blockDim.x) {
        stage_row64(base + OFF_W1, r, m.w16 + MLP_H_W1 + r * 16, 2);
        stage_row64(base + OFF_W2, r, m.w16 + MLP_H_W2 + r * 64, 8);
        stage_row64(base + OFF_W3, r, m.w16 + MLP_H_W3 + r * 64, 8);
    }
    for (int i = tid; i < 256; i += blockDim.x) {
        float v;
        if (i < 64) v = m.params[MLP_B1 + i];
        else if (i < 128) v = m.params[MLP_B2 + i - 64];
        else if (i < 192) v = m.params[MLP_B3 + i - 128];
        else v = __half2float(m.w16[MLP_H_W4 + (i - 192)]);
        sBias[i] = v;
    }
    if (tid == 0) {
        sBias[256] = m.params[MLP_B4];
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, TC_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t tmem_warp = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t a_addr = tc::smem_addr(act);
    const float b4 = sBias[256];
    const float amb = tp.ambient;
    const unsigned total = *sb.flat_total;
    const unsigned ntiles = (total + 127u) / 128u;
    unsigned phase = 0, n_fallback = 0, n_valid = 0;
    bool failed = false;

    // the current row: slot, position + weight, light; its features
    unsigned tile = blockIdx.x;
    size_t idx = 0;
    bool valid = tile < ntiles && locate(sb, tile * 128u + tid, total, idx);
    float4 s = valid ? sb.pos_w[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    float g = valid ? sb.light_lane[idx].x : 0.f;
    uint32_t xin[8];
    bool fb = false;
    auto featurize = [&](const float4& sp, bool v, uint32_t (&x)[8], bool& out_fb) {
        if (v) {
            float f[MLP_IN];
            mlp::features<FMT, true>(vd, m, sp.x, sp.y, sp.z, tp.sun[0], tp.sun[1], tp.sun[2],
                                     f);
            out_fb = !mlp::in_range(m, f);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                x[q] = mlp::pack_h2((f[2 * q] - m.mu[2 * q]) * m.inv_sd[2 * q],
                                    (f[2 * q + 1] - m.mu[2 * q + 1]) * m.inv_sd[2 * q + 1]);
        } else {
            out_fb = false;
#pragma unroll
            for (int q = 0; q < 8; ++q) x[q] = 0u;
        }
    };
    featurize(s, valid, xin, fb);

    for (; tile < ntiles; tile += gridDim.x) {
        // ---- A. the tile's inputs -> layer 1
        *reinterpret_cast<uint4*>(act + tc::sw128_offset(tid, 0)) =
            make_uint4(xin[0], xin[1], xin[2], xin[3]);
        *reinterpret_cast<uint4*>(act + tc::sw128_offset(tid, 1)) =
            make_uint4(xin[4], xin[5], xin[6], xin[7]);
        // ---- B. the next tile's row: slot and sample loads (consumed in D)
        const unsigned ntile = tile + gridDim.x;
        size_t nidx = 0;
        const bool nvalid = ntile < ntiles && locate(sb, ntile * 128u + tid, total, nidx);
        float4 ns = make_float4(0.f, 0.f, 0.f, 0.f);
        float ng = 0.f;
        if (nvalid) {
            ns = sb.pos_w[nidx];
            ng = sb.light_lane[nidx].x;
        }
        uint32_t nx[8];
        bool nfb = false;
        float y = 0.f;
#pragma unroll 1
        for (int layer = 0; layer < 3; ++layer) {
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
                const uint32_t w_addr = tc::smem_addr(base + OFF_W1 + 8192 * layer);
                const int ksteps = layer == 0 ? 1 : 4;
                for (int k = 0; k < ksteps; ++k)
                    tc::mma_f16(tmem, tc::desc_sw128(a_addr + 32u * k),
                                tc::desc_sw128(w_addr + 32u * k), IDESC, k > 0 ? 1u : 0u);
                tc::mma_commit(bar);
            }
            // ---- D. while layer 2 runs: the next chunk's features
            if (layer == 1) featurize(ns, nvalid, nx, nfb);
            const bool ok = tc::mbar_wait(bar, phase, TC_WAIT_LIMIT);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
            // ---- C/E. epilogue: TMEM -> registers -> bias + SiLU, 32 columns
            // at a time; the last layer folds the 64 -> 1 output in FP32
            float yy = b4;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                uint32_t acc[32];
                tc::tmem_ld32(tmem_warp + 32u * half, acc);
                uint32_t h[16];
                bias_silu32(acc, sBias + 64 * layer + 32 * half, h);
                if (layer < 2) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<uint4*>(act + tc::sw128_offset(tid, 4 * half + q)) =
                            make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
                } else {
                    const float* w4 = sBias + 192 + 32 * half;
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const float2 v =
                            __half22float2(*reinterpret_cast<const __half2*>(&h[q]));
                        yy = fmaf(w4[2 * q], v.x, yy);
                        yy = fmaf(w4[2 * q + 1], v.y, yy);
                    }
                }
            }
            if (layer == 2) y = yy;
            tc::fence_before_sync();
        }
        if (failed) break;
        if (valid) {
            n_valid++;
            float tau;
            if (fb) {
                tau = cgs::sun_cone<FMT>(vd, cone, s.x, s.y, s.z, tp.sun[0], tp.sun[1],
                                         tp.sun[2]);
                n_fallback++;
            } else {
                tau = m.tau_scale * mlp::softplus(y);
            }
            sb.pos_w[idx].w = s.w * __expf(-tp.sigma * tau) * (amb + (1.f - amb) * g);
        }
        // ---- G. advance
        valid = nvalid;
        idx = nidx;
        s = ns;
        g = ng;
        fb = nfb;
#pragma unroll
        for (int q = 0; q < 8; ++q) xin[q] = nx[q];
    }
    if (failed) {
        // drain the outstanding commit (bounded), then report
        tc::mbar_wait(bar, phase, TC_WAIT_LIMIT);
        if (tid == 0) atomicOr(status + 1, 1ull);
    }
    unsigned tot = n_fallback, nv = n_valid;
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        nv += __shfl_xor_sync(0xffffffffu, nv, o);
    }
    if (lane == 0) {
        if (tot) atomicAdd(status, (unsigned long long)tot);
        if (nv) atomicAdd(status + 2, (unsigned long long)nv);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

}  // namespace

cudaError_t launch_shade_mlp_tc(VolDesc vd, CamDesc cam, TraceParams tp, const MlpDev& m,
                                SampleBuf sb, unsigned long long* status, cudaStream_t st) {
    ConeSchedule cone = make_cone_schedule(vd, tp);
    static bool configured[2][64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const int f = vd.fmt == 0 ? 0 : 1;
    if (!configured[f][dev]) {
        e = f == 0 ? cudaFuncSetAttribute(k_shade_mlp_tc<0>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES)
                   : cudaFuncSetAttribute(k_shade_mlp_tc<1>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        configured[f][dev] = true;
    }
    (void)cam;
    // 4 resident CTAs per SM (shared memory and 4 x 64 tensor-memory columns)
    const int blocks = 152 * 4;
    if (f == 0)
        k_shade_mlp_tc<0><<<blocks, 128, SMEM_BYTES, st>>>(vd, tp, cone, m, sb, status);
    else
        k_shade_mlp_tc<1><<<blocks, 128, SMEM_BYTES, st>>>(vd, tp, cone, m, sb, status);
    return cudaGetLastError();
}
