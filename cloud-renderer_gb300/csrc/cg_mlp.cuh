// cg_mlp.cuh -- the sun-transmittance surrogate: 16 features -> 3 x 64 SiLU
// -> 1 (normalized optical depth).  FP16 weights and activations on the tensor
// cores (mma.sync m16n8k16, FP32 accumulation), FP32 master weights for Adam.
#pragma once

#include <cuda_fp16.h>

#include "cg_internal.h"
#include "cg_sample.cuh"

// (layout constants and MlpDev: cg_internal.h)
// padded shared-memory row strides (halfs): conflict-free ldmatrix rows
#define MLP_S16 24
#define MLP_S64 72
#define MLP_SMEM_W_HALFS (64 * MLP_S16 + 2 * 64 * MLP_S64 + 8 * MLP_S64)

namespace mlp {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                        uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1,
                                          uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

// D = A * B + D, m16n8k16, f16 inputs, f32 accumulators.
__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Output link: tau = tau_scale * softplus(y) keeps the predicted optical depth
// positive and the transmittance exp(-sigma tau) in (0, 1].
__device__ __forceinline__ float softplus(float y) {
    return fmaxf(y, 0.f) + __logf(1.f + __expf(-fabsf(y)));
}
__device__ __forceinline__ float sigmoid(float y) { return 1.f / (1.f + __expf(-y)); }

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }

// SiLU on two FP16 values: silu(z) = h (1 + tanh h), h = z / 2 -- one MUFU
// tanh for two activations.  Used by every forward pass (training and
// inference alike).
__device__ __forceinline__ uint32_t silu_h2(uint32_t z) {
    uint32_t h, t, r;
    const uint32_t half2_05 = 0x38003800u;  // (0.5, 0.5)
    asm("mul.rn.f16x2 %0, %1, %2;" : "=r"(h) : "r"(z), "r"(half2_05));
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.f16x2 %0, %1, %2, %1;" : "=r"(r) : "r"(h), "r"(t));
    return r;
}
__device__ __forceinline__ float silu_grad(float z) {
    float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// Copy the FP16 weight image into padded shared memory (all threads of the CTA).
__device__ __forceinline__ void load_weights(const __half* w16, __half* sW) {
    for (int i = threadIdx.x; i < MLP_NHALF; i += blockDim.x) {
        __half v = w16[i];
        int dst;
        if (i < MLP_H_W2) {
            dst = (i / 16) * MLP_S16 + (i % 16);
        } else if (i < MLP_H_W3) {
            int j = i - MLP_H_W2;
            dst = 64 * MLP_S16 + (j / 64) * MLP_S64 + (j % 64);
        } else if (i < MLP_H_W4) {
            int j = i - MLP_H_W3;
            dst = 64 * MLP_S16 + 64 * MLP_S64 + (j / 64) * MLP_S64 + (j % 64);
        } else {
            int j = i - MLP_H_W4;
            dst = 64 * MLP_S16 + 2 * 64 * MLP_S64 + (j / 64) * MLP_S64 + (j % 64);
        }
        sW[dst] = v;
    }
}

__device__ __forceinline__ const __half* sw1(const __half* sW) { return sW; }
__device__ __forceinline__ const __half* sw2(const __half* sW) { return sW + 64 * MLP_S16; }
__device__ __forceinline__ const __half* sw3(const __half* sW) {
    return sW + 64 * MLP_S16 + 64 * MLP_S64;
}
__device__ __forceinline__ const __half* sw4(const __half* sW) {
    return sW + 64 * MLP_S16 + 2 * 64 * MLP_S64;
}

// Accumulator tiles (8 n-tiles of a 16-row block) -> A fragments of the next
// layer (4 k-slices): the m16n8 C layout of two adjacent n-tiles is the m16k16
// A layout.
__device__ __forceinline__ void acc_to_a(const float acc[8][4], uint32_t a[4][4]) {
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        a[ks][0] = pack_h2(acc[2 * ks][0], acc[2 * ks][1]);
        a[ks][1] = pack_h2(acc[2 * ks][2], acc[2 * ks][3]);
        a[ks][2] = pack_h2(acc[2 * ks + 1][0], acc[2 * ks + 1][1]);
        a[ks][3] = pack_h2(acc[2 * ks + 1][2], acc[2 * ks + 1][3]);
    }
}

// acc[nt] = bias (columns 8nt + 2t, +1) + A(16 x 64) * W^T for one 64-wide layer.
__device__ __forceinline__ void layer64(const uint32_t a[4][4], const __half* sWl,
                                        const float* bias, float acc[8][4]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
        acc[nt][0] = b0;
        acc[nt][1] = b1;
        acc[nt][2] = b0;
        acc[nt][3] = b1;
    }
#pragma unroll
    for (int np = 0; np < 4; ++np) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int n = np * 16 + (lane & 7) + (lane >> 4) * 8;
            const int k = ks * 16 + ((lane >> 3) & 1) * 8;
            uint32_t b0, b1, b2, b3;
            ldsm_x4(smem_u32(sWl + n * MLP_S64 + k), b0, b1, b2, b3);
            mma16816(acc[2 * np], a[ks], b0, b1);
            mma16816(acc[2 * np + 1], a[ks], b2, b3);
        }
    }
}

// Forward of one 16-row block whose normalised FP16 inputs are rows [0,16)
// of sX (stride MLP_S16).  Returns y for rows g and g+8 in lanes with t == 0.
// If zs is given, the pre-activations of layers 1-3 are stored there (FP16,
// [16][MLP_S64] each) for the backward pass.
__device__ __forceinline__ void forward16(const __half* sX, const __half* sW, const float* b1,
                                          const float* b2, const float* b3, float b4,
                                          float& y_g, float& y_g8, __half* z1 = nullptr,
                                          __half* z2 = nullptr, __half* z3 = nullptr,
                                          __half* h1 = nullptr, __half* h2 = nullptr) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t ax[4];
    {
        const int r = (lane & 7) + ((lane >> 3) & 1) * 8;
        const int c = (lane >> 4) * 8;
        ldsm_x4(smem_u32(sX + r * MLP_S16 + c), ax[0], ax[1], ax[2], ax[3]);
    }
    float acc[8][4];
    // layer 1: K = 16
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float bb0 = b1[8 * nt + 2 * t], bb1 = b1[8 * nt + 2 * t + 1];
        acc[nt][0] = bb0;
        acc[nt][1] = bb1;
        acc[nt][2] = bb0;
        acc[nt][3] = bb1;
    }
#pragma unroll
    for (int np = 0; np < 4; ++np) {
        const int n = np * 16 + (lane & 7) + (lane >> 4) * 8;
        const int k = ((lane >> 3) & 1) * 8;
        uint32_t w0, w1, w2, w3;
        ldsm_x4(smem_u32(sw1(sW) + n * MLP_S16 + k), w0, w1, w2, w3);
        mma16816(acc[2 * np], ax, w0, w1);
        mma16816(acc[2 * np + 1], ax, w2, w3);
    }
    __half* zs[3] = {z1, z2, z3};
    __half* hs[2] = {h1, h2};
    const float* bs[2] = {b2, b3};
    const __half* ws[2] = {sw2(sW), sw3(sW)};
    uint32_t a[4][4];
    // a[ks][0..3] hold (row g | g+8, cols 16ks + 2t | 16ks + 8 + 2t) pairs
    auto store = [&](__half* dst, const uint32_t (&v)[4][4]) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int c0 = 16 * ks + 2 * t, c1 = c0 + 8;
            *reinterpret_cast<uint32_t*>(dst + g * MLP_S64 + c0) = v[ks][0];
            *reinterpret_cast<uint32_t*>(dst + (g + 8) * MLP_S64 + c0) = v[ks][1];
            *reinterpret_cast<uint32_t*>(dst + g * MLP_S64 + c1) = v[ks][2];
            *reinterpret_cast<uint32_t*>(dst + (g + 8) * MLP_S64 + c1) = v[ks][3];
        }
    };
#pragma unroll
    for (int layer = 0; layer < 3; ++layer) {
        acc_to_a(acc, a);  // pre-activations, FP16
        if (zs[layer]) store(zs[layer], a);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks)
#pragma unroll
            for (int e = 0; e < 4; ++e) a[ks][e] = silu_h2(a[ks][e]);
        if (layer < 2 && hs[layer]) store(hs[layer], a);
        if (layer < 2) layer64(a, ws[layer], bs[layer], acc);
    }
    // output layer: W4 rows 1-7 are zero, column 0 is the result
    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        // one n-tile: x2 would suffice; x4 with the same rows keeps one helper
        const int n = (lane & 7);
        const int k = ks * 16 + ((lane >> 3) & 1) * 8;
        uint32_t w0, w1, w2, w3;
        ldsm_x4(smem_u32(sw4(sW) + n * MLP_S64 + k), w0, w1, w2, w3);
        mma16816(o, a[ks], w0, w1);
    }
    y_g = o[0] + b4;
    y_g8 = o[2] + b4;
}

// Forward of 32 rows (rows [0,32) of sX): both 16-row blocks advance layer by
// layer together so that every weight fragment loaded from shared memory
// feeds two MMAs.  y[0] holds rows g, g+8 and y[1] rows 16+g, 24+g, valid in
// lanes with t == 0.
__device__ __forceinline__ void forward32(const __half* sX, const __half* sW, const float* b1,
                                          const float* b2, const float* b3, float b4,
                                          float y[2][2]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    uint32_t a[2][4][4];
    float acc[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        uint32_t ax[4];
        const int r = mt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
        const int c = (lane >> 4) * 8;
        ldsm_x4(smem_u32(sX + r * MLP_S16 + c), ax[0], ax[1], ax[2], ax[3]);
#pragma unroll
        for (int e = 0; e < 4; ++e) a[mt][0][e] = ax[e];
    }
    // layer 1 (K = 16)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bb0 = b1[8 * nt + 2 * t], bb1 = b1[8 * nt + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc[mt][nt][0] = bb0;
            acc[mt][nt][1] = bb1;
            acc[mt][nt][2] = bb0;
            acc[mt][nt][3] = bb1;
        }
    }
#pragma unroll
    for (int np = 0; np < 4; ++np) {
        const int n = np * 16 + (lane & 7) + (lane >> 4) * 8;
        const int k = ((lane >> 3) & 1) * 8;
        uint32_t w0, w1, w2, w3;
        ldsm_x4(smem_u32(sw1(sW) + n * MLP_S16 + k), w0, w1, w2, w3);
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            mma16816(acc[mt][2 * np], a[mt][0], w0, w1);
            mma16816(acc[mt][2 * np + 1], a[mt][0], w2, w3);
        }
    }
    const float* bs[2] = {b2, b3};
    const __half* ws[2] = {sw2(sW), sw3(sW)};
#pragma unroll
    for (int layer = 0; layer < 3; ++layer) {
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc_to_a(acc[mt], a[mt]);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
#pragma unroll
                for (int e = 0; e < 4; ++e) a[mt][ks][e] = silu_h2(a[mt][ks][e]);
        }
        if (layer == 2) break;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float bb0 = bs[layer][8 * nt + 2 * t], bb1 = bs[layer][8 * nt + 2 * t + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                acc[mt][nt][0] = bb0;
                acc[mt][nt][1] = bb1;
                acc[mt][nt][2] = bb0;
                acc[mt][nt][3] = bb1;
            }
        }
#pragma unroll
        for (int np = 0; np < 4; ++np) {
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const int n = np * 16 + (lane & 7) + (lane >> 4) * 8;
                const int k = ks * 16 + ((lane >> 3) & 1) * 8;
                uint32_t b0, b1r, b2r, b3r;
                ldsm_x4(smem_u32(ws[layer] + n * MLP_S64 + k), b0, b1r, b2r, b3r);
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    mma16816(acc[mt][2 * np], a[mt][ks], b0, b1r);
                    mma16816(acc[mt][2 * np + 1], a[mt][ks], b2r, b3r);
                }
            }
        }
    }
    float o[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        const int n = (lane & 7);
        const int k = ks * 16 + ((lane >> 3) & 1) * 8;
        uint32_t w0, w1, w2, w3;
        ldsm_x4(smem_u32(sw4(sW) + n * MLP_S64 + k), w0, w1, w2, w3);
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) mma16816(o[mt], a[mt][ks], w0, w1);
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        y[mt][0] = o[mt][0] + b4;
        y[mt][1] = o[mt][2] + b4;
    }
}

// Features of one query (see MlpDev, FeatGeom): the 12 density taps are
// filtered by the texture unit (training and inference share this function).
__device__ __forceinline__ void features(const FeatGeom& g, float vx, float vy, float vz,
                                         float sx, float sy, float sz, float f[MLP_IN]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float X = vx * g.sc[i], Y = vy * g.sc[i], Z = vz * g.sc[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float d = g.dsc[3 * i + k];
            // the texture returns exactly 0 on an empty footprint: no
            // occupancy branch, so the 12 fetches issue back to back
            f[3 * i + k] = tex3D<float2>((cudaTextureObject_t)g.tex[i], fmaf(d, sx, X),
                                         fmaf(d, sy, Y), fmaf(d, sz, Z))
                               .x;
        }
    }
    f[12] = vx * g.invD;
    f[13] = vy * g.invD;
    f[14] = vz * g.invD;
    f[15] = sy;
}

__device__ __forceinline__ bool in_range(const MlpDev& m, const float f[MLP_IN]) {
    bool ok = true;
#pragma unroll
    for (int j = 0; j < MLP_IN; ++j) ok = ok && (f[j] >= m.fmin[j]) && (f[j] <= m.fmax[j]);
    return ok;
}

}  // namespace mlp
