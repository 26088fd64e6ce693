// k_textures.cu -- hardware-filtered copies of the pyramid and the noise
// lattices for the approximate (surrogate) renderer.
//
// The exact path interpolates in software because the texture unit's 8-bit
// filter weights cannot meet a 1e-4 bound.  The surrogate path is held to an
// image RMSE of 1e-2 instead, so it lets the texture units do the trilinear
// filtering: each level is copied into a 3D array of half2 (density, light)
// with border addressing (outside reads 0) and linear filtering, and each
// noise octave's lattice table into a 3D float array.  Value noise with
// smoothstep weights is one hardware trilinear fetch at the smoothstep-warped
// coordinate.
#include "cg_internal.h"
#include "cg_sample.cuh"

namespace {

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }

template <int FMT>
__global__ void k_pack_level(VolDesc vd, int l, cudaSurfaceObject_t surf) {
    const int N = vd.dims[l];
    const long long total = (long long)N * N * N;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((long long)N * N));
        const long long idx = vd.offs[l] + i;
        float r, g;
        if (FMT == 0) {
            float4 v = reinterpret_cast<const float4*>(vd.pyr)[idx];
            r = v.x;
            g = v.y;
        } else {
            uint32_t v = reinterpret_cast<const uint32_t*>(vd.pyr)[idx];
            r = bf16_lo(v);
            g = __half2float(__ushort_as_half((unsigned short)(v >> 16)));
        }
        __half2 h = __floats2half2_rn(r, g);
        surf3Dwrite(*reinterpret_cast<uint32_t*>(&h), surf, x * 4, y, z);
    }
}

// fBm at the texel centres of an R^3 grid over the noise domain (origin org,
// extent ext per axis), in noise coordinates (no further shift).
__global__ void k_fbm_volume(TraceParams tp, float ox, float oy, float oz, float ex, float ey,
                             float ez, int R, cudaSurfaceObject_t surf) {
    const long long total = (long long)R * R * R;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        const float qx = ox + ((float)x + 0.5f) / (float)R * ex;
        const float qy = oy + ((float)y + 0.5f) / (float)R * ey;
        const float qz = oz + ((float)z + 0.5f) / (float)R * ez;
        __half h = __float2half_rn(cgs::fbm_q(tp, qx, qy, qz));
        surf3Dwrite(__half_as_ushort(h), surf, x * 2, y, z);
    }
}

}  // namespace

cudaError_t launch_fbm_volume(TraceParams tp, const float org[3], const float ext[3], int R,
                              cudaSurfaceObject_t surf, cudaStream_t st) {
    const long long total = (long long)R * R * R;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_fbm_volume<<<blocks, 256, 0, st>>>(tp, org[0], org[1], org[2], ext[0], ext[1], ext[2], R,
                                         surf);
    return cudaGetLastError();
}

cudaError_t launch_pack_level(VolDesc vd, int l, cudaSurfaceObject_t surf, cudaStream_t st) {
    const long long N = vd.dims[l];
    const long long total = N * N * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (vd.fmt == 0)
        k_pack_level<0><<<blocks, 256, 0, st>>>(vd, l, surf);
    else
        k_pack_level<1><<<blocks, 256, 0, st>>>(vd, l, surf);
    return cudaGetLastError();
}

CG_OOB_TU(k_textures)
