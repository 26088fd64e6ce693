// cg_check.cuh -- the bounds-check build.  Built with CG_BOUNDS_CHECK=1 (see
// build.py: a separate library, libcloudgb_check.so), the hot kernels test
// the global-memory indexes they compute -- pyramid and occupancy gathers,
// sample-record and contribution scatters, voxel stores -- against the size
// of the buffer: an index out of range skips the access and is recorded in
// the translation unit's error word (a count and the first offending source
// line and index), never a trap.  cg_bounds_violations() collects and clears
// the words of every translation unit.  In the normal build the checks are
// the constant true and compile away.
#pragma once

#include <cuda_runtime.h>

#ifndef CG_BOUNDS_CHECK
#define CG_BOUNDS_CHECK 0
#endif

#if defined(__CUDACC__) && CG_BOUNDS_CHECK
// [0] violations, [1] (source line << 32) | low 32 bits of the first bad index
static __device__ unsigned long long cg_oob_word[2];

__device__ __forceinline__ bool cg_in_bounds(unsigned long long i, unsigned long long n,
                                             unsigned line) {
    if (i < n) return true;
    if (atomicAdd(&cg_oob_word[0], 1ull) == 0ull)
        cg_oob_word[1] = ((unsigned long long)line << 32) | (i & 0xFFFFFFFFull);
    return false;
}
#define CG_IN_BOUNDS(i, n) cg_in_bounds((unsigned long long)(i), (unsigned long long)(n), __LINE__)
// The translation unit's reader: copies its word to out and clears it.
#define CG_OOB_TU(name)                                                                 \
    cudaError_t cg_oob_take_##name(unsigned long long out[2]) {                        \
        cudaError_t e = cudaMemcpyFromSymbol(out, cg_oob_word, sizeof(cg_oob_word));    \
        if (e != cudaSuccess) return e;                                                 \
        const unsigned long long zero[2] = {0ull, 0ull};                                \
        return cudaMemcpyToSymbol(cg_oob_word, zero, sizeof(zero));                     \
    }
#elif defined(__CUDACC__)
#define CG_IN_BOUNDS(i, n) true
#define CG_OOB_TU(name)                                            \
    cudaError_t cg_oob_take_##name(unsigned long long out[2]) {   \
        out[0] = out[1] = 0ull;                                   \
        return cudaSuccess;                                       \
    }
#endif

// Total violations of every translation unit since the last call (cleared);
// site receives "<file>:<line> index <i>" of the first one found.  Always 0
// outside the bounds-check build.
unsigned long long cg_bounds_take(char* site, int site_len, cudaError_t* err);
