// cg_mlp_tc.cuh -- the surrogate network (16 -> 64 [-> 64 [-> 64]] SiLU -> 1:
// one to three hidden layers) on the fifth-generation tensor cores, shared by
// the shade kernel, the standalone inference kernel (k_shade_tc.cu) and the
// fused renderer (k_render_tc.cu): the weight tiles a CTA stages in shared
// memory, one layer's MMA issue, and one layer's epilogue for a thread's row.
//
// Network tiles of a layout for up to NL hidden layers (Net<NL>; bytes from
// a 1024-aligned base, Net<NL>::BYTES in all):
//   W2, W3   64 x 128 B, 128B-swizzled K-major (K = 64), present for NL >= 2, 3
//   W1       64 x 32 B, 32B-swizzled (K = 16)
//   ONES     one 8-row 32B-swizzled atom, every row (1, 1, 0, ...)
//   BIAS     NL x (64 x 32 B) 32B-swizzled: row n = (b_hi[n], b_lo[n], 0, ...)
// Layers 1-3 run on weights and biases pre-scaled by 1/2 (exact in FP16 and
// FP32), so the accumulator holds z/2 and SiLU is z/2 * (1 + tanh(z/2)).  The
// bias enters as one more K = 16 MMA: the ones column against the bias split
// into two FP16 halves (exact to ~2^-22 relative).  An activation tile is 128
// rows x 128 B, 128B-swizzled; its first 32 B of a row hold the 16 inputs.
#pragma once

#include <cuda_fp16.h>

#include "cg_internal.h"
#include "cg_mlp.cuh"
#include "cg_tc.cuh"

namespace mlptc {

template <int NL>
struct Net {
    static constexpr int W2 = 0;
    static constexpr int W3 = 8192;
    static constexpr int W1 = 8192 * (NL - 1);
    static constexpr int ONES = W1 + 2048;
    static constexpr int BIAS = ONES + 256;
    static constexpr int BYTES = BIAS + NL * 2048;
    static_assert(NL >= 1 && NL <= MLP_MAX_LAYERS, "hidden layers");
    static_assert(W1 % 256 == 0 && ONES % 256 == 0 && BIAS % 256 == 0, "SW32 alignment");
};
constexpr int ACT_BYTES = 128 * 128;  // one activation tile

constexpr uint32_t IDESC = tc::idesc_f16_f32(128, 64);

// One FP16 weight row (`chunks` x 8 halves) into row r of a swizzled tile
// (128B-swizzled rows of 8 chunks, or 32B-swizzled rows of 2), scaled by 1/2.
template <int CHUNKS>
__device__ __forceinline__ void stage_row(uint8_t* tile, int r, const __half* src) {
    const __half2 k = __floats2half2_rn(0.5f, 0.5f);
#pragma unroll
    for (int c = 0; c < CHUNKS; ++c) {
        uint4 v = *reinterpret_cast<const uint4*>(src + 8 * c);
        __half2* h = reinterpret_cast<__half2*>(&v);
#pragma unroll
        for (int q = 0; q < 4; ++q) h[q] = __hmul2(h[q], k);
        *reinterpret_cast<uint4*>(tile + (CHUNKS == 8 ? tc::sw128_offset(r, c)
                                                      : tc::sw32_offset(r, c))) = v;
    }
}

// The model's hidden-layer weights (W1 .. W_layers, m.layers <= NL) scaled by
// 1/2, the ones column (8 rows) and the split half-scaled biases into the
// Net<NL> tiles at `net`; threads t = 0 .. n-1.
template <int NL>
__device__ __forceinline__ void stage_network(uint8_t* net, const MlpDev& m, int t, int n) {
    using L = Net<NL>;
    for (int r = t; r < 64; r += n) {
        stage_row<2>(net + L::W1, r, m.w16 + MLP_H_W1 + r * 16);
        if (NL >= 2 && m.layers >= 2) stage_row<8>(net + L::W2, r, m.w16 + MLP_H_W2 + r * 64);
        if (NL >= 3 && m.layers >= 3) stage_row<8>(net + L::W3, r, m.w16 + MLP_H_W3 + r * 64);
    }
    if (t < 8) {
        const __half one = __float2half_rn(1.f);
        const uint32_t ones =
            (uint32_t)__half_as_ushort(one) | ((uint32_t)__half_as_ushort(one) << 16);
        *reinterpret_cast<uint4*>(net + L::ONES + tc::sw32_offset(t, 0)) =
            make_uint4(ones, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(net + L::ONES + tc::sw32_offset(t, 1)) =
            make_uint4(0u, 0u, 0u, 0u);
    }
    for (int i = t; i < m.layers * 64; i += n) {
        const int l = i >> 6, r = i & 63;
        const float hb = m.k.hb[i];
        const __half hi = __float2half_rn(hb);
        const __half lo = __float2half_rn(hb - __half2float(hi));
        uint8_t* tile = net + L::BIAS + 2048 * l;
        *reinterpret_cast<uint4*>(tile + tc::sw32_offset(r, 0)) = make_uint4(
            (uint32_t)__half_as_ushort(hi) | ((uint32_t)__half_as_ushort(lo) << 16), 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(tile + tc::sw32_offset(r, 1)) = make_uint4(0u, 0u, 0u, 0u);
    }
}

// Issue one layer (one thread) into tensor memory at d_tmem and commit it to
// `bar`: the K slices of the activation tile at a_addr against the layer's
// weights (Net<NL> tiles at net_addr), then the bias slice.  The ones operand
// is a single 8-row atom read by all 16 row groups (stride byte offset 0).
template <int NL>
__device__ __forceinline__ void issue_layer(int layer, uint32_t d_tmem, uint32_t a_addr,
                                            uint32_t net_addr, uint64_t* bar) {
    using L = Net<NL>;
    if (layer == 0) {
        tc::mma_f16(d_tmem, tc::desc_sw128(a_addr), tc::desc_sw32(net_addr + L::W1), IDESC, 0u);
    } else {
        const uint32_t w_addr = net_addr + (layer == 1 ? L::W2 : L::W3);
        for (int k = 0; k < 4; ++k)
            tc::mma_f16(d_tmem, tc::desc_sw128(a_addr + 32u * k),
                        tc::desc_sw128(w_addr + 32u * k), IDESC, k > 0 ? 1u : 0u);
    }
    tc::mma_f16(d_tmem, tc::desc_sw32(net_addr + L::ONES, 0u),
                tc::desc_sw32(net_addr + L::BIAS + 2048u * layer), IDESC, 1u);
    tc::mma_commit(bar);
}

// SiLU of 32 half-scaled accumulators (the bias is already in them) -> 16
// FP16 pairs: with h = z/2, silu(z) = h + h * tanh(h), evaluated in FP32 and
// rounded once.
__device__ __forceinline__ void silu32(const uint32_t (&acc)[32], uint32_t (&out)[16]) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float a = __uint_as_float(acc[2 * j]);
        const float b = __uint_as_float(acc[2 * j + 1]);
        float ta, tb;
        asm("tanh.approx.f32 %0, %1;" : "=f"(ta) : "f"(a));
        asm("tanh.approx.f32 %0, %1;" : "=f"(tb) : "f"(b));
        out[j] = mlp::pack_h2(fmaf(a, ta, a), fmaf(b, tb, b));
    }
}

// One layer's epilogue for tile row `row` (this thread's tensor-memory lane,
// dw = the lane's address of the layer's 64 accumulator columns): SiLU, 32
// columns at a time, written as the next layer's FP16 activations, or, for
// the last hidden layer, folded into the FP32 64 -> 1 output (returned with b4).
__device__ __forceinline__ float layer_epilogue(bool last, uint32_t dw, uint8_t* act, int row,
                                                const MlpDev& m) {
    float yy = m.k.b4;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        uint32_t acc[32];
        tc::tmem_ld32(dw + 32u * half, acc);
        uint32_t h[16];
        silu32(acc, h);
        if (!last) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                *reinterpret_cast<uint4*>(act + tc::sw128_offset(row, 4 * half + q)) =
                    make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
        } else {
            const float* w4 = m.k.w4 + 32 * half;
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const float2 v = __half22float2(*reinterpret_cast<const __half2*>(&h[q]));
                yy = fmaf(w4[2 * q], v.x, yy);
                yy = fmaf(w4[2 * q + 1], v.y, yy);
            }
        }
    }
    return yy;
}

// The normalised FP16 inputs of a row (features f) into chunks 0-1 of
// activation-tile row `row`; zeros for an empty row.
__device__ __forceinline__ void write_inputs(uint8_t* act, int row, const MlpDev& m,
                                             const float (&f)[MLP_IN], bool valid) {
    uint32_t x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        x[q] = valid ? mlp::pack_h2((f[2 * q] - m.mu[2 * q]) * m.inv_sd[2 * q],
                                    (f[2 * q + 1] - m.mu[2 * q + 1]) * m.inv_sd[2 * q + 1])
                     : 0u;
    *reinterpret_cast<uint4*>(act + tc::sw128_offset(row, 0)) = make_uint4(x[0], x[1], x[2], x[3]);
    *reinterpret_cast<uint4*>(act + tc::sw128_offset(row, 1)) = make_uint4(x[4], x[5], x[6], x[7]);
}

}  // namespace mlptc
