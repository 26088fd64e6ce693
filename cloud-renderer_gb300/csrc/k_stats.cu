// k_stats.cu -- image error statistics reduced on the GPU in FP64: the one
// place FP64 arithmetic runs on the device (the render path itself is FP32).
//
// Per RGBA channel: max |a - ref| and the sum of squared differences, over n
// pixels of a (FP32) against ref (FP64 or FP32).  Two passes with fixed
// reduction orders (per-CTA partials, then one CTA), so results do not depend
// on scheduling.
#include "cg_internal.h"

namespace {

constexpr int STATS_CTAS = 152 * 4;
constexpr int STATS_THREADS = 256;

template <typename R>
__global__ void __launch_bounds__(STATS_THREADS) k_err_partials(const float4* a, const R* ref,
                                                                size_t n, double* part) {
    double mx[4] = {0, 0, 0, 0}, ss[4] = {0, 0, 0, 0};
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = a[i];
        const double av[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const double d = av[c] - (double)ref[4 * i + c];
            mx[c] = fmax(mx[c], fabs(d));
            ss[c] += d * d;
        }
    }
    __shared__ double sm[STATS_THREADS][8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        sm[threadIdx.x][c] = mx[c];
        sm[threadIdx.x][4 + c] = ss[c];
    }
    __syncthreads();
    for (int s = STATS_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                sm[threadIdx.x][c] = fmax(sm[threadIdx.x][c], sm[threadIdx.x + s][c]);
                sm[threadIdx.x][4 + c] += sm[threadIdx.x + s][4 + c];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 8) part[(size_t)blockIdx.x * 8 + threadIdx.x] = sm[0][threadIdx.x];
}

__global__ void __launch_bounds__(STATS_THREADS) k_err_final(const double* part, int nparts,
                                                             double* out) {
    __shared__ double sm[STATS_THREADS][8];
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < nparts; p += blockDim.x)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            v[c] = fmax(v[c], part[(size_t)p * 8 + c]);
            v[4 + c] += part[(size_t)p * 8 + 4 + c];
        }
#pragma unroll
    for (int c = 0; c < 8; ++c) sm[threadIdx.x][c] = v[c];
    __syncthreads();
    for (int s = STATS_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                sm[threadIdx.x][c] = fmax(sm[threadIdx.x][c], sm[threadIdx.x + s][c]);
                sm[threadIdx.x][4 + c] += sm[threadIdx.x + s][4 + c];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 8) out[threadIdx.x] = sm[0][threadIdx.x];
}

}  // namespace

size_t err_stats_scratch_bytes() { return (size_t)STATS_CTAS * 8 * sizeof(double) + 64; }

cudaError_t launch_err_stats(const float4* a, const void* ref, int ref_f64, size_t n,
                             double* scratch, double* out, cudaStream_t st) {
    if (ref_f64)
        k_err_partials<double><<<STATS_CTAS, STATS_THREADS, 0, st>>>(
            a, reinterpret_cast<const double*>(ref), n, scratch);
    else
        k_err_partials<float><<<STATS_CTAS, STATS_THREADS, 0, st>>>(
            a, reinterpret_cast<const float*>(ref), n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_err_final<<<1, STATS_THREADS, 0, st>>>(scratch, STATS_CTAS, out);
    return cudaGetLastError();
}

CG_OOB_TU(k_stats)
