// k_mlp.cu -- the sun-transmittance surrogate's kernels: feature extraction,
// inference, the fused training step (forward + backward, tensor cores) and
// the gradient reduction with Adam.
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

// ---- training step -----------------------------------------------------------------
// One CTA = 128 rows (4 warps x 2 blocks of 16).  Loss per row:
//   (exp(-sigma * tau_scale * softplus(y)) - exp(-sigma * tau))^2,
// the per-row gradient is written without the 1/batch factor (applied in
// the reduction) to keep FP16 intermediates away from underflow.  Every CTA
// writes its full gradient (and loss sum) to its own slot of `partial`.
struct TrainSmem {
    // offsets in halfs from the start of dynamic shared memory
    static constexpr int W = 0;
    static constexpr int X = W + MLP_SMEM_W_HALFS;
    static constexpr int Z1 = X + 128 * MLP_S16;
    static constexpr int Z2 = Z1 + 128 * MLP_S64;
    static constexpr int Z3 = Z2 + 128 * MLP_S64;
    static constexpr int H1 = Z3 + 128 * MLP_S64;
    static constexpr int H2 = H1 + 128 * MLP_S64;
    static constexpr int D1 = H2 + 128 * MLP_S64;
    static constexpr int D2 = D1 + 128 * MLP_S64;
    static constexpr int D3 = D2 + 128 * MLP_S64;
    static constexpr int HALF_END = D3 + 128 * MLP_S64;
    // floats after the halfs
    static constexpr int F_BIAS = 0;           // b1 b2 b3 b4 (193)
    static constexpr int F_DY = 196;           // 128
    static constexpr int F_TAU = F_DY + 128;   // 128
    static constexpr int F_RED = F_TAU + 128;  // [4 layers][4 warps][64]
    static constexpr int F_LOSS = F_RED + 4 * 4 * 64;  // [4] loss, [4] db4 per warp
    static constexpr int FLOAT_END = F_LOSS + 8;
    static constexpr size_t BYTES = (size_t)HALF_END * 2 + (size_t)FLOAT_END * 4;
};

// dH(16 x 64) = dZ(16 x 64, A fragments) * W (W stored [out][in]; B via .trans)
__device__ __forceinline__ void layer64_bwd(const uint32_t a[4][4], const __half* sWl,
                                            float acc[8][4]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int np = 0; np < 4; ++np) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int row = ks * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;  // out index
            const int col = np * 16 + (lane >> 4) * 8;                     // in index
            uint32_t b0, b1, b2, b3;
            ldsm_x4_t(smem_u32(sWl + row * MLP_S64 + col), b0, b1, b2, b3);
            mma16816(acc[2 * np], a[ks], b0, b1);
            mma16816(acc[2 * np + 1], a[ks], b2, b3);
        }
    }
}

// Multiply the accumulators by silu'(z) (z FP16 rows g, g+8 of a 16-row block),
// store them as FP16 dZ, add their column sums to colsum[16] (cols 8nt+2t, +1).
__device__ __forceinline__ void apply_silu_grad(float acc[8][4], const __half* z, __half* dz,
                                                float colsum[16]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int c = 8 * nt + 2 * t;
        float2 za = __half22float2(*reinterpret_cast<const __half2*>(z + g * MLP_S64 + c));
        float2 zb = __half22float2(*reinterpret_cast<const __half2*>(z + (g + 8) * MLP_S64 + c));
        acc[nt][0] *= silu_grad(za.x);
        acc[nt][1] *= silu_grad(za.y);
        acc[nt][2] *= silu_grad(zb.x);
        acc[nt][3] *= silu_grad(zb.y);
        *reinterpret_cast<__half2*>(dz + g * MLP_S64 + c) = __floats2half2_rn(acc[nt][0], acc[nt][1]);
        *reinterpret_cast<__half2*>(dz + (g + 8) * MLP_S64 + c) =
            __floats2half2_rn(acc[nt][2], acc[nt][3]);
        colsum[2 * nt] += acc[nt][0] + acc[nt][2];
        colsum[2 * nt + 1] += acc[nt][1] + acc[nt][3];
    }
}

// Reduce per-lane column sums over the 8 lanes sharing t; lanes 0-3 write
// columns 8nt+2t, +1 of `dst` (64 floats).
__device__ __forceinline__ void store_colsum(float colsum[16], float* dst) {
    const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float v = colsum[j];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        colsum[j] = v;
    }
    if (lane < 4) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            dst[8 * nt + 2 * t] = colsum[2 * nt];
            dst[8 * nt + 2 * t + 1] = colsum[2 * nt + 1];
        }
    }
}

// dW[out][in] (16 outs = m-tile mt, NT n-tiles of 8 ins) = sum over 128 rows of
// dZ[row][out] * A[row][in]; dZ, A FP16 in shared memory.
template <int NT, int SA>
__device__ __forceinline__ void weight_grad(const __half* dZ, const __half* A, int mtile,
                                            float acc[NT][4]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const int m0 = mtile * 16;
#pragma unroll
    for (int ks = 0; ks < 8; ++ks) {
        const int k0 = ks * 16;
        uint32_t a[4];
        {
            const int row = k0 + (lane & 7) + (lane >> 4) * 8;
            const int col = m0 + ((lane >> 3) & 1) * 8;
            ldsm_x4_t(smem_u32(dZ + row * MLP_S64 + col), a[0], a[1], a[2], a[3]);
        }
#pragma unroll
        for (int np = 0; np < NT / 2; ++np) {
            const int row = k0 + (lane & 7) + ((lane >> 3) & 1) * 8;
            const int col = np * 16 + (lane >> 4) * 8;
            uint32_t b0, b1, b2, b3;
            ldsm_x4_t(smem_u32(A + row * SA + col), b0, b1, b2, b3);
            mma16816(acc[2 * np], a, b0, b1);
            mma16816(acc[2 * np + 1], a, b2, b3);
        }
    }
}

__global__ void __launch_bounds__(128) k_mlp_train(TrainArgs ta) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half* hs = reinterpret_cast<__half*>(smem);
    float* fs = reinterpret_cast<float*>(smem + (size_t)TrainSmem::HALF_END * 2);
    __half* sW = hs + TrainSmem::W;
    __half* sX = hs + TrainSmem::X;
    float* sB = fs + TrainSmem::F_BIAS;
    float* sDy = fs + TrainSmem::F_DY;
    float* sTau = fs + TrainSmem::F_TAU;
    float* sRed = fs + TrainSmem::F_RED;
    float* sLoss = fs + TrainSmem::F_LOSS;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;

    load_weights(ta.w16, sW);
    for (int i = tid; i < 3 * 64 + 1; i += blockDim.x)
        sB[i] = i < 64 ? ta.params[MLP_B1 + i]
                       : (i < 128 ? ta.params[MLP_B2 + i - 64]
                                  : (i < 192 ? ta.params[MLP_B3 + i - 128] : ta.params[MLP_B4]));
    // batch rows: sequential (gradient evaluation) or a multiplicative
    // permutation of the dataset that advances with the step counter
    {
        const long long r = (long long)blockIdx.x * 128 + tid;
        bool valid;
        long long idx;
        if (ta.sequential) {
            idx = ta.offset + r;
            valid = idx < ta.N;
        } else {
            const long long step = ta.step ? *ta.step : 0;
            const unsigned long long lin = (unsigned long long)(step * ta.batch + r);
            idx = (long long)((lin * ta.perm_mul) % (unsigned long long)ta.N);
            valid = true;
        }
#pragma unroll
        for (int j = 0; j < MLP_IN; ++j) {
            float f = valid ? ta.feat[(size_t)idx * MLP_IN + j] : 0.f;
            sX[tid * MLP_S16 + j] = __float2half_rn((f - ta.mu[j]) * ta.inv_sd[j]);
        }
        sTau[tid] = valid ? ta.tau[idx] : -1.f;  // < 0 marks a padding row
    }
    __syncthreads();

    // forward (two 16-row blocks per warp) and the output gradient
    float loss = 0.f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int base = w * 32 + mt * 16;
        float yg, yg8;
        forward16(sX + base * MLP_S16, sW, sB, sB + 64, sB + 128, sB[192], yg, yg8,
                  hs + TrainSmem::Z1 + base * MLP_S64, hs + TrainSmem::Z2 + base * MLP_S64,
                  hs + TrainSmem::Z3 + base * MLP_S64, hs + TrainSmem::H1 + base * MLP_S64,
                  hs + TrainSmem::H2 + base * MLP_S64);
        if (t == 0) {
            const float k = ta.sigma * ta.tau_scale;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = base + g + 8 * h;
                const float y = h ? yg8 : yg;
                const float tau = sTau[row];
                float dy = 0.f;
                if (tau >= 0.f) {
                    const float Th = __expf(-k * softplus(y)), T = __expf(-ta.sigma * tau);
                    const float diff = Th - T;
                    loss += diff * diff;
                    dy = 2.f * diff * (-k * sigmoid(y) * Th);
                }
                sDy[row] = dy;
            }
        }
    }
    __syncwarp();
    loss += __shfl_xor_sync(0xffffffffu, loss, 4);
    loss += __shfl_xor_sync(0xffffffffu, loss, 8);
    loss += __shfl_xor_sync(0xffffffffu, loss, 16);
    if (lane == 0) sLoss[w] = loss;

    // backward through the layers, per 16-row block
    float cs4[16], cs3[16], cs2[16], cs1[16], db4 = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) cs4[j] = cs3[j] = cs2[j] = cs1[j] = 0.f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int base = w * 32 + mt * 16;
        const __half* z3 = hs + TrainSmem::Z3 + base * MLP_S64;
        const float dyg = sDy[base + g], dyg8 = sDy[base + g + 8];
        if (t == 0) db4 += dyg + dyg8;
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = 8 * nt + 2 * t;
            const float w4a = __half2float(sw4(sW)[c]), w4b = __half2float(sw4(sW)[c + 1]);
            float2 za = __half22float2(*reinterpret_cast<const __half2*>(z3 + g * MLP_S64 + c));
            float2 zb =
                __half22float2(*reinterpret_cast<const __half2*>(z3 + (g + 8) * MLP_S64 + c));
            // dW4 column sums: silu(z3) * dy
            cs4[2 * nt] += silu(za.x) * dyg + silu(zb.x) * dyg8;
            cs4[2 * nt + 1] += silu(za.y) * dyg + silu(zb.y) * dyg8;
            acc[nt][0] = dyg * w4a;
            acc[nt][1] = dyg * w4b;
            acc[nt][2] = dyg8 * w4a;
            acc[nt][3] = dyg8 * w4b;
        }
        apply_silu_grad(acc, z3, hs + TrainSmem::D3 + base * MLP_S64, cs3);
        uint32_t a[4][4];
        acc_to_a(acc, a);
        layer64_bwd(a, sw3(sW), acc);
        apply_silu_grad(acc, hs + TrainSmem::Z2 + base * MLP_S64,
                        hs + TrainSmem::D2 + base * MLP_S64, cs2);
        acc_to_a(acc, a);
        layer64_bwd(a, sw2(sW), acc);
        apply_silu_grad(acc, hs + TrainSmem::Z1 + base * MLP_S64,
                        hs + TrainSmem::D1 + base * MLP_S64, cs1);
    }
    store_colsum(cs4, sRed + (0 * 4 + w) * 64);
    store_colsum(cs3, sRed + (1 * 4 + w) * 64);
    store_colsum(cs2, sRed + (2 * 4 + w) * 64);
    store_colsum(cs1, sRed + (3 * 4 + w) * 64);
    db4 += __shfl_xor_sync(0xffffffffu, db4, 4);
    db4 += __shfl_xor_sync(0xffffffffu, db4, 8);
    db4 += __shfl_xor_sync(0xffffffffu, db4, 16);
    if (lane == 0) sLoss[4 + w] = db4;
    __syncthreads();

    float* part = ta.partial + (size_t)blockIdx.x * (MLP_NPARAM + 1);
    // biases, dW4 and the loss: fixed-order sums over the 4 warps
    if (tid < 64) {
        const int c = tid;
        float s4 = 0.f, s3 = 0.f, s2 = 0.f, s1 = 0.f;
#pragma unroll
        for (int ww = 0; ww < 4; ++ww) {
            s4 += sRed[(0 * 4 + ww) * 64 + c];
            s3 += sRed[(1 * 4 + ww) * 64 + c];
            s2 += sRed[(2 * 4 + ww) * 64 + c];
            s1 += sRed[(3 * 4 + ww) * 64 + c];
        }
        part[MLP_W4 + c] = s4;
        part[MLP_B3 + c] = s3;
        part[MLP_B2 + c] = s2;
        part[MLP_B1 + c] = s1;
    }
    if (tid == 0) {
        part[MLP_B4] = ((sLoss[4] + sLoss[5]) + sLoss[6]) + sLoss[7];
        part[MLP_NPARAM] = ((sLoss[0] + sLoss[1]) + sLoss[2]) + sLoss[3];
    }
    // weight gradients: warp w owns output rows 16w..16w+15 of each layer
    {
        float acc[8][4];
        weight_grad<8, MLP_S64>(hs + TrainSmem::D3, hs + TrainSmem::H2, w, acc);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int o = 16 * w + g, i = 8 * nt + 2 * t;
            part[MLP_W3 + o * 64 + i] = acc[nt][0];
            part[MLP_W3 + o * 64 + i + 1] = acc[nt][1];
            part[MLP_W3 + (o + 8) * 64 + i] = acc[nt][2];
            part[MLP_W3 + (o + 8) * 64 + i + 1] = acc[nt][3];
        }
        weight_grad<8, MLP_S64>(hs + TrainSmem::D2, hs + TrainSmem::H1, w, acc);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int o = 16 * w + g, i = 8 * nt + 2 * t;
            part[MLP_W2 + o * 64 + i] = acc[nt][0];
            part[MLP_W2 + o * 64 + i + 1] = acc[nt][1];
            part[MLP_W2 + (o + 8) * 64 + i] = acc[nt][2];
            part[MLP_W2 + (o + 8) * 64 + i + 1] = acc[nt][3];
        }
        float acc1[2][4];
        weight_grad<2, MLP_S16>(hs + TrainSmem::D1, sX, w, acc1);
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int o = 16 * w + g, i = 8 * nt + 2 * t;
            part[MLP_W1 + o * 16 + i] = acc1[nt][0];
            part[MLP_W1 + o * 16 + i + 1] = acc1[nt][1];
            part[MLP_W1 + (o + 8) * 16 + i] = acc1[nt][2];
            part[MLP_W1 + (o + 8) * 16 + i + 1] = acc1[nt][3];
        }
    }
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
__global__ void k_mlp_adam(AdamArgs aa) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int step = aa.step ? *aa.step : 0;
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

cudaError_t launch_mlp_train(const TrainArgs& ta, int ctas, cudaStream_t st) {
    // the attribute is set once per device, outside any stream capture
    static std::atomic<bool> configured[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!configured[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)TrainSmem::BYTES);
        if (e != cudaSuccess) return e;
        configured[dev].store(true, std::memory_order_release);
    }
    k_mlp_train<<<ctas, 128, TrainSmem::BYTES, st>>>(ta);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const AdamArgs& aa, cudaStream_t st) {
    k_mlp_adam<<<(MLP_NPARAM + 1 + 255) / 256, 256, 0, st>>>(aa);
    return cudaGetLastError();
}
