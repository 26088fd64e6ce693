// cg_mlp.cuh -- the sun-transmittance surrogate's shared device helpers: the
// 16 input features of a sample, their trained range, FP16 packing and the
// output link.  The network itself (16 -> 3 x 64 SiLU -> 1, FP16 operands,
// FP32 accumulation) runs on the tensor cores in k_shade_tc.cu (inference)
// and k_train_tc.cu (training); FP32 master weights live with Adam.
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

}  // namespace mlp
