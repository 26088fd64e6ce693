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

// Sum the CTA gradients in CTA order, scale by 1/batch, Adam update (or just
// return the gradient).  The last CTA to finish advances the step counter.
// A training kernel that stopped on a bounded wait (non-zero status) leaves
// stale or half-written partials: no update then, and the step stays.
__global__ void k_mlp_adam(AdamArgs aa) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int step = aa.step ? *aa.step : 0;
    if (aa.status && *aa.status) {
        if (p == MLP_NPARAM) adam_param(aa, p, step, true);  // the NaN loss slot
        return;
    }
    if (p <= MLP_NPARAM) adam_param(aa, p, step, false);
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
