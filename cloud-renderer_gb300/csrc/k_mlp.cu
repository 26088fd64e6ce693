// k_mlp.cu -- the sun-transmittance surrogate's feature extraction and the
// gradient reduction with Adam (the network's forward and backward passes run
// on the tensor cores in k_shade_tc.cu and k_train_tc.cu).
#include <atomic>

#include "cg_mlp.cuh"

namespace {

using namespace mlp;

// ---- features ----------------------------------------------------------------
__global__ void k_mlp_features(FeatGeom g, const float* pos, int n, float sx, float sy, float sz,
                               float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[MLP_IN];
    features(g, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], sx, sy, sz, f);
#pragma unroll
    for (int j = 0; j < MLP_IN; ++j) out[(size_t)i * MLP_IN + j] = f[j];
}

// Index of parameter p in the FP16 weight image (-1 for biases).
__device__ __forceinline__ int half_index(int p) {
    if (p < MLP_B1) return MLP_H_W1 + p;
    if (p >= MLP_W2 && p < MLP_B2) return MLP_H_W2 + (p - MLP_W2);
    if (p >= MLP_W3 && p < MLP_B3) return MLP_H_W3 + (p - MLP_W3);
    if (p >= MLP_W4 && p < MLP_B4) return MLP_H_W4 + (p - MLP_W4);
    return -1;
}

// Sum the CTA gradients in CTA order, scale by 1/batch, Adam update (or just
// return the gradient).  The last CTA to finish advances the step counter.
// A training kernel that stopped on a bounded wait (non-zero status) leaves
// stale or half-written partials: no update then, and the step stays.
__global__ void k_mlp_adam(AdamArgs aa) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int step = aa.step ? *aa.step : 0;
    if (aa.status && *aa.status) {
        if (p == MLP_NPARAM && aa.loss_out)
            aa.loss_out[aa.loss_slot_by_step ? step - aa.loss_base : 0] = __int_as_float(0x7fc00000);
        return;
    }
    if (p <= MLP_NPARAM) {
        float g = 0.f;
        for (int c = 0; c < aa.nparts; ++c) g += aa.partial[(size_t)c * (MLP_NPARAM + 1) + p];
        g *= aa.inv_batch;
        if (p == MLP_NPARAM) {
            if (aa.loss_out) aa.loss_out[aa.loss_slot_by_step ? step - aa.loss_base : 0] = g;
        } else if (aa.grad_out) {
            aa.grad_out[p] = g;
        } else {
            const float t1 = (float)(step + 1);
            float m = aa.m[p] = aa.beta1 * aa.m[p] + (1.f - aa.beta1) * g;
            float v = aa.v[p] = aa.beta2 * aa.v[p] + (1.f - aa.beta2) * g * g;
            const float mh = m / (1.f - powf(aa.beta1, t1));
            const float vh = v / (1.f - powf(aa.beta2, t1));
            const float w = aa.params[p] - aa.lr * mh / (sqrtf(vh) + aa.eps);
            aa.params[p] = w;
            const int hi = half_index(p);
            if (hi >= 0) aa.w16[hi] = __float2half_rn(w);
        }
    }
    if (aa.step && !aa.grad_out) {
        __shared__ bool last;
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) last = atomicAdd(aa.ticket, 1u) == gridDim.x - 1;
        __syncthreads();
        if (last && threadIdx.x == 0) {
            *aa.ticket = 0u;
            *aa.step = step + 1;
        }
    }
}

}  // namespace

cudaError_t launch_mlp_features(VolDesc vd, const MlpDev& m, const float* pos, int n,
                                const float dir[3], float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_mlp_features<<<(n + 127) / 128, 128, 0, st>>>(feat_geom(vd, m), pos, n, dir[0], dir[1],
                                                    dir[2], out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const AdamArgs& aa, cudaStream_t st) {
    k_mlp_adam<<<(MLP_NPARAM + 1 + 255) / 256, 256, 0, st>>>(aa);
    return cudaGetLastError();
}

CG_OOB_TU(k_mlp)
