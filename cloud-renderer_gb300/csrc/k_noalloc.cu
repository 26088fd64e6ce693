// k_noalloc.cu -- cg_sun_map_noalloc: the sun-view nearest-surface map and
// its highlight stores for callers that cannot allocate device memory.
//
// Who needs it: hosts that own every byte of device memory themselves
// (engines with a fixed budget carved out at start-up, plugin hosts whose
// allocator must not be bypassed) and real-time threads that cannot afford
// cudaMalloc's implicit device synchronisation in the middle of a frame.
// cg_voxelize keeps its per-texel depth keys in memory owned by the volume;
// this entry point keeps them in a fixed array compiled into the library, so
// the call itself allocates nothing: the caller passes the boards and the two
// outputs, all in device memory.
//
// The scratch array below is CG_NOALLOC_MAX_TEXELS 64-bit keys (8 MiB).  Every
// GPU that loads the library holds it until the process exits.  All calls on a
// device share it: calls whose work overlaps on the GPU (different streams,
// or different host threads) race on it, so serialise them.
#include <cstdio>
#include <mutex>

#include "cg_internal.h"
#include "cloudgb.h"

static __device__ __align__(256) unsigned long long g_noalloc_keys[CG_NOALLOC_MAX_TEXELS];

namespace {

// Device address of g_noalloc_keys per device.  In host code the symbol names
// a host-side stand-in, not device memory, so the address is looked up once
// per device with that device current and cached.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long* g_keys_addr[kMaxDevices] = {};

cudaError_t keys_for_current_device(unsigned long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_keys_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_keys);
        if (e != cudaSuccess) return e;
        g_keys_addr[dev] = reinterpret_cast<unsigned long long*>(p);
    }
    *out = g_keys_addr[dev];
    return cudaSuccess;
}

cg_status noalloc_fail(cg_status s, const char* msg) {
    char buf[256];
    snprintf(buf, sizeof(buf), "cg_sun_map_noalloc: %s", msg);
    set_last_error(buf);
    return s;
}

}  // namespace

extern "C" cg_status cg_sun_map_noalloc(int dimension, float bound_min, float bound_max,
                                        const float position[3], const float* d_boards,
                                        int count, const cg_sun* sun, float* d_positions,
                                        uint8_t* d_mask, void* stream) {
    if (!position || !sun || !d_positions || !d_mask || (count > 0 && !d_boards))
        return noalloc_fail(CG_ERR_INVALID_ARGUMENT, "null pointer");
    if (dimension < 2 || dimension > 512)
        return noalloc_fail(CG_ERR_OUT_OF_RANGE, "dimension not in [2, 512]");
    if (count < 0 || count > (1 << 24))
        return noalloc_fail(CG_ERR_OUT_OF_RANGE, "count not in [0, 2^24]");
    if (!(bound_max > bound_min)) return noalloc_fail(CG_ERR_INVALID_ARGUMENT, "bounds");
    const long long texels = (long long)sun->map_width * sun->map_height;
    if (sun->map_width < 1 || sun->map_height < 1 || texels > CG_NOALLOC_MAX_TEXELS)
        return noalloc_fail(CG_ERR_OUT_OF_RANGE,
                            "sun map must hold between 1 and CG_NOALLOC_MAX_TEXELS "
                            "(1048576) texels");
    SunFrame fr;
    if (!sun_frame_for_box(position, bound_min, bound_max, sun->direction, sun->map_width,
                           sun->map_height, fr))
        return noalloc_fail(CG_ERR_INVALID_ARGUMENT,
                            "sun direction is zero or parallel to the up axis (0,1,0)");
    unsigned long long* keys = nullptr;
    cudaError_t e = keys_for_current_device(&keys);
    if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // World box and highlight offset exactly as cg_voxelize derives them.
    float wmin[3], range[3];
    for (int a = 0; a < 3; ++a) {
        wmin[a] = position[a] + bound_min;
        range[a] = (position[a] + bound_max) - wmin[a];
    }
    float vs0 = range[0] / (float)dimension, vs1 = range[1] / (float)dimension,
          vs2 = range[2] / (float)dimension;
    float step = vs0 < vs1 ? vs0 : vs1;
    step = step < vs2 ? step : vs2;
    const float offset = step * 0.57735026f;
    // The shared array keeps the previous call's keys: reset them to "empty",
    // and clear the caller's mask (stores only ever set bytes to 1).
    e = cudaMemsetAsync(keys, 0xFF, (size_t)texels * 8, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_mask, 0, (size_t)dimension * dimension * dimension, s);
    if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, cudaGetErrorString(e));
    BoardsDev b{};
    b.n = count;
    b.cwr = reinterpret_cast<const float4*>(d_boards);
    if (count > 0) {
        e = launch_sunmap(b, fr, reinterpret_cast<uint64_t*>(keys), s);
        if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, cudaGetErrorString(e));
    }
    e = launch_highlight(b, fr, reinterpret_cast<const uint64_t*>(keys),
                         reinterpret_cast<float4*>(d_positions), dimension, wmin, range, offset,
                         d_mask, nullptr, s);
    if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, cudaGetErrorString(e));
    return CG_OK;
}

CG_OOB_TU(k_noalloc)
