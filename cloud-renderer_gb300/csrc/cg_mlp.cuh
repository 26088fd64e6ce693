// cg_mlp.cuh -- the sun-transmittance surrogate's shared device helpers: the
// 16 input features of a sample, their trained range, FP16 packing, the
// output link and the per-parameter optimiser step.  The network itself
// (16 -> 1..3 x 64 SiLU -> 1, FP16 operands, FP32 accumulation) runs on the
// tensor cores in k_shade_tc.cu / k_render_tc.cu (inference) and
// k_train_tc.cu (training); FP32 master weights live with Adam.
#pragma once

#include <cuda_fp16.h>

#include "cg_internal.h"
#include "cg_sample.cuh"

// (layout constants and MlpDev: cg_internal.h)

namespace mlp {

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

// Index of parameter p in the FP16 weight image (-1 for biases).
__device__ __forceinline__ int half_index(int p) {
    if (p < MLP_B1) return MLP_H_W1 + p;
    if (p >= MLP_W2 && p < MLP_B2) return MLP_H_W2 + (p - MLP_W2);
    if (p >= MLP_W3 && p < MLP_B3) return MLP_H_W3 + (p - MLP_W3);
    if (p >= MLP_W4 && p < MLP_B4) return MLP_H_W4 + (p - MLP_W4);
    return -1;
}

// Parameter p (p == MLP_NPARAM: the loss) of one optimiser step: the CTA
// partials summed in CTA order and scaled by 1/batch, then the loss slot, the
// returned gradient, or the Adam update of the FP32 master, its moments and
// its FP16 copy.  The separate optimiser kernel and the training kernel's
// fused tail both call it, so the two give bit-identical steps.  stopped: a
// training kernel stopped on a bounded wait (non-zero status) and left stale
// or half-written partials -- the loss slot is NaN and nothing is updated.
// The partials are read past L1 (other SMs wrote them in the same launch when
// the optimiser is fused).
__device__ __forceinline__ void adam_param(const AdamArgs& aa, int p, int step, bool stopped) {
    if (stopped) {
        if (p == MLP_NPARAM && aa.loss_out)
            aa.loss_out[aa.loss_slot_by_step ? step - aa.loss_base : 0] = __int_as_float(0x7fc00000);
        return;
    }
    if (p >= aa.frozen_lo && p < aa.frozen_hi) {  // a hidden layer the model does not use
        if (aa.grad_out) aa.grad_out[p] = 0.f;
        return;
    }
    // explicit roundings (no FMA contraction left to the compiler): the two
    // kernels that inline this must issue the same operations
    // CTA order, sixteen loads in flight at a time
    const float* src = aa.partial + p;
    constexpr size_t STRIDE = MLP_NPARAM + 1;
    float g = 0.f;
    int c = 0;
    for (; c + 16 <= aa.nparts; c += 16) {
        float v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) v[u] = __ldcg(src + (size_t)(c + u) * STRIDE);
#pragma unroll
        for (int u = 0; u < 16; ++u) g = __fadd_rn(g, v[u]);
    }
    for (; c < aa.nparts; ++c) g = __fadd_rn(g, __ldcg(src + (size_t)c * STRIDE));
    g = __fmul_rn(g, aa.inv_batch);
    if (p == MLP_NPARAM) {
        if (aa.loss_out) aa.loss_out[aa.loss_slot_by_step ? step - aa.loss_base : 0] = g;
    } else if (aa.grad_out) {
        aa.grad_out[p] = g;
    } else {
        const float t1 = (float)(step + 1);
        const float m = __fmaf_rn(aa.beta1, aa.m[p], __fmul_rn(__fsub_rn(1.f, aa.beta1), g));
        const float v = __fmaf_rn(aa.beta2, aa.v[p],
                                  __fmul_rn(__fmul_rn(__fsub_rn(1.f, aa.beta2), g), g));
        aa.m[p] = m;
        aa.v[p] = v;
        const float mh = __fdiv_rn(m, __fsub_rn(1.f, powf(aa.beta1, t1)));
        const float vh = __fdiv_rn(v, __fsub_rn(1.f, powf(aa.beta2, t1)));
        const float w = __fsub_rn(aa.params[p], __fdiv_rn(__fmul_rn(aa.lr, mh),
                                                          __fadd_rn(__fsqrt_rn(vh), aa.eps)));
        aa.params[p] = w;
        const int hi = half_index(p);
        if (hi >= 0) aa.w16[hi] = __float2half_rn(w);
    }
}

}  // namespace mlp
