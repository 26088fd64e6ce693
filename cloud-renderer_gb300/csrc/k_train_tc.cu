// k_train_tc.cu -- one training step of the sun-transmittance surrogate on the
// fifth-generation tensor cores: forward, loss gradient, backward and the
// per-CTA gradient partials that k_mlp_adam reduces in a fixed order.
//
// One CTA = 128 rows of the batch, 16 warps: four threads per row, each on 16
// of the 64 columns of every epilogue (warps w, w + 4, w + 8, w + 12 share the
// tensor-memory lanes 32 (w % 4) ..).  The network has NL = 1, 2 or 3 hidden
// layers (a template parameter).  Every GEMM is a
// tcgen05.mma (M = 128, FP16 operands from shared memory, FP32 accumulators
// in tensor memory) issued by thread 0 and committed to one mbarrier:
//   forward   z_l = A_l W_l^T + b_l          A_0 = x, A_l = h_l (K = 16, 64)
//   backward  dh_l = dz_{l+1} W_{l+1}        (A = dz rows, B = W^T rows)
//             [dW_l | db_l] = dz_l^T [h_l | 1] (A = dz^T, padded to 128 rows;
//             B = h^T plus a row of ones: the bias gradient is column 64 of
//             the same product; K = the 128 batch rows)
// Pre-activations are kept in FP16 (z_h) and SiLU is evaluated in FP32 on
// them; activations and gradients enter the MMAs as FP16.  The output layer
// (64 -> 1) and its gradients are FP32: each thread's share of the output dot,
// summed over the four parts in part order, and dW4 by deterministic
// warp-shuffle trees.  Transposed operands (dz^T, h^T, x^T) are written by the
// threads that own the rows and columns.  Every mbarrier wait is bounded (ta.wait_ns
// of the global timer, 1 s in training); a timeout sets the status word (and
// partial[NPARAM] to NaN), drains, frees tensor memory and returns: k_mlp_adam
// then makes no update and the host reports CG_ERR_DEVICE_FAULT.
//
// Fused optimiser (ta.grid_bar set, cooperative launch): the step is one
// launch.  After its partials every CTA arrives at a grid barrier and each
// then reduces and updates a slice of the parameters with the same function,
// in the same CTA order, as k_mlp_adam -- the two paths give identical bits.
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>

#include "cg_internal.h"
#include "cg_mlp.cuh"
#include "cg_tc.cuh"

namespace {

constexpr uint32_t TT_COLS = 256;  // [0, 64) forward / dh, [64, 160) dW | db
// four threads per batch row, each on 16 of the 64 columns of every epilogue
// (16 warps: four per tensor-memory lane quarter)
constexpr int TT_PARTS = 4;
constexpr int TT_THREADS = 128 * TT_PARTS;
constexpr int CW = 64 / TT_PARTS;
static_assert(CW == 16, "ld_cols loads 16 columns");
constexpr int ZS = 66;  // halves per row of the z stores (conflict-free rows)
// shared memory map (bytes from the 1024-aligned base)
constexpr int O_X = 0;             // 128 x 128 B SW128 (K = 16 used)
constexpr int O_H1 = 16384;        // 128 x 128 B SW128
constexpr int O_H2 = 32768;        // 128 x 128 B SW128
constexpr int O_D = 49152;         // 128 x 128 B SW128: dz rows
constexpr int O_DT = 65536;        // 2 K-atoms x 128 rows x 128 B: dz^T (rows 64-127 zero)
constexpr int DT_ATOM = 16384;
constexpr int O_HT = 98304;        // 2 K-atoms x 80 rows x 128 B: h^T / x^T, row 64 = ones
constexpr int HT_ATOM = 10240;
constexpr int O_W1 = O_HT + 2 * HT_ATOM;  // 64 x 32 B SW32 (K = 16)
constexpr int O_W2 = O_W1 + 2048;  // 64 x 128 B SW128
constexpr int O_W3 = O_W2 + 8192;
constexpr int O_WT2 = O_W3 + 8192;  // W2^T: row = input, K = output
constexpr int O_WT3 = O_WT2 + 8192;
constexpr int O_ONES = O_WT3 + 8192;  // one 8-row SW32 atom: rows (1, 1, 0, ...)
constexpr int O_BIAS = O_ONES + 256;  // 3 x (64 x 32 B) SW32: (b_hi, b_lo, 0, ...)
constexpr int O_Z = O_BIAS + 3 * 2048;           // 3 x 128 x ZS halves
// floats: dy[128], w4[64], red[4][64], misc[16], output partials [TT_PARTS][128]
constexpr int O_F = O_Z + 3 * 128 * ZS * 2;
constexpr int O_BAR = O_F + (128 + 64 + 4 * 64 + 16 + TT_PARTS * 128) * 4;
constexpr int TT_USED = O_BAR + 32;
constexpr int TT_SMEM = TT_USED + 1024;
static_assert(O_W2 % 1024 == 0 && O_W3 % 1024 == 0 && O_WT2 % 1024 == 0 && O_WT3 % 1024 == 0 &&
                  O_HT % 1024 == 0 && O_DT % 1024 == 0 && HT_ATOM % 1024 == 0,
              "128B-swizzled tiles need 1024-byte alignment");
static_assert(O_ONES % 256 == 0 && O_BIAS % 256 == 0 && O_W1 % 256 == 0, "SW32 alignment");
static_assert(TT_SMEM <= 227 * 1024, "shared memory");

constexpr uint32_t ID64 = tc::idesc_f16_f32(128, 64);
constexpr uint32_t ID80 = tc::idesc_f16_f32(128, 80);

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

// byte address of element (row, k) of a 128B-swizzled K-major tile whose
// K-atoms (64 halves each) are `atom` bytes apart
__device__ __forceinline__ uint32_t kt_addr(int row, int k, int atom) {
    return (uint32_t)((k >> 6) * atom) + tc::sw128_offset(row, (k & 63) >> 3) + (uint32_t)((k & 7) * 2);
}

__device__ __forceinline__ void mma_k(uint32_t d, uint32_t a, uint32_t b, uint32_t id, int ksteps,
                                      int a_atom, int b_atom, bool acc0) {
    for (int k = 0; k < ksteps; ++k) {
        const uint32_t off = 32u * (k & 3);
        tc::mma_f16(d, tc::desc_sw128(a + (uint32_t)((k >> 2) * a_atom) + off),
                    tc::desc_sw128(b + (uint32_t)((k >> 2) * b_atom) + off), id,
                    (acc0 || k > 0) ? 1u : 0u);
    }
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad_f(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// sync + the CTA's agreement on a failed wait
__device__ __forceinline__ bool tt_sync(bool bad) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    const bool any_bad = __syncthreads_or(bad) != 0;
    tc::fence_after_sync();
    return any_bad;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The optimiser tail of a fused step.  Each CTA's partials, its reads of the
// step counter and of the weights all come before its arrival at the grid
// barrier, every update after the last arrival.  The barrier is a monotonic
// arrival counter: a completed step leaves it at a multiple of gridDim.x, so
// the generation of an arrival is its ticket / gridDim.x.  Its wait is bounded
// by four mbarrier limits -- longer than the slowest CTA that still arrives
// (a wait that ran out plus its drain) -- and sets status bit 2 when it runs
// out; a CTA that failed a wait set its bit before arriving, so after the
// barrier every CTA sees it and no slice is updated.
__device__ void fused_adam(const TrainArgs& ta, int step, int* flag) {
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned ticket = atomicAdd(ta.grid_bar, 1u);
        const unsigned target = (ticket / gridDim.x + 1u) * gridDim.x;
        const uint64_t limit = 4ull * ta.wait_ns, t0 = tc::global_ns();
        bool met = true;
        while (ld_acquire(ta.grid_bar) < target) {
            if (tc::global_ns() - t0 > limit) {
                met = false;
                break;
            }
            __nanosleep(32);
        }
        if (!met) atomicOr(ta.status, 4ull);
        __threadfence();
        *flag = *reinterpret_cast<volatile unsigned long long*>(ta.status) != 0ull ? 1 : 0;
    }
    __syncthreads();
    const bool stopped = *flag != 0;
    // 128 parameters per CTA (the first four warps), so that the slices spread
    // over as many SMs as there are
    if (threadIdx.x < 128)
        for (int p = blockIdx.x * 128 + threadIdx.x; p <= MLP_NPARAM; p += gridDim.x * 128)
            mlp::adam_param(ta.adam, p, step, stopped);
    if (blockIdx.x == 0 && threadIdx.x == 0 && !stopped) *ta.adam.step = step + 1;
}

// CW FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void ld_cols(uint32_t taddr, float (&v)[CW]) {
    uint32_t r[16];
    tc::tmem_ld16(taddr, r);
#pragma unroll
    for (int j = 0; j < CW; ++j) v[j] = __uint_as_float(r[j]);
}

template <int NL>
__global__ void __launch_bounds__(TT_THREADS, 1) k_mlp_train_tc(TrainArgs ta) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_addr(smem_raw);
    uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t sb = tc::smem_addr(base);
    __half* zs = reinterpret_cast<__half*>(base + O_Z);
    float* fdy = reinterpret_cast<float*>(base + O_F);
    float* fw4 = fdy + 128;
    float* fred = fw4 + 64;
    float* fmisc = fred + 4 * 64;
    float* fyp = fmisc + 16;  // [TT_PARTS][128] partial output dots
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + O_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + O_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // thread = (row, part): the row's tensor-memory lane is row (warp w reads
    // lanes 32 (w % 4) ..), the part its CW columns c0 .. c0 + CW - 1
    const int row = tid & 127, part = tid >> 7, wq = warp & 3;
    const int c0 = part * CW;

    // ---- weights (FP16 image) of the NL hidden layers, the transposes of
    // layers 2 .. NL, biases, ones
    for (int i = tid; i < 64 * 2; i += TT_THREADS) {
        const int r = i >> 1, c = i & 1;
        *reinterpret_cast<uint4*>(base + O_W1 + tc::sw32_offset(r, c)) =
            *reinterpret_cast<const uint4*>(ta.w16 + MLP_H_W1 + r * 16 + 8 * c);
    }
#pragma unroll
    for (int l = 1; l < NL; ++l) {
        const int src = l == 1 ? MLP_H_W2 : MLP_H_W3;
        uint8_t* w = base + (l == 1 ? O_W2 : O_W3);
        uint8_t* wt = base + (l == 1 ? O_WT2 : O_WT3);
        for (int i = tid; i < 64 * 8; i += TT_THREADS) {
            const int r = i >> 3, c = i & 7;
            *reinterpret_cast<uint4*>(w + tc::sw128_offset(r, c)) =
                *reinterpret_cast<const uint4*>(ta.w16 + src + r * 64 + 8 * c);
            // W^T row r (input r), K = outputs 8c .. 8c+7
            __align__(16) __half t[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) t[q] = ta.w16[src + (8 * c + q) * 64 + r];
            *reinterpret_cast<uint4*>(wt + tc::sw128_offset(r, c)) =
                *reinterpret_cast<const uint4*>(t);
        }
    }
    for (int r = tid; r < 64; r += TT_THREADS) fw4[r] = __half2float(ta.w16[MLP_H_W4 + r]);
    for (int i = tid; i < NL * 64; i += TT_THREADS) {
        const int l = i >> 6, n = i & 63;
        const int off = l == 0 ? MLP_B1 : (l == 1 ? MLP_B2 : MLP_B3);
        const float bv = ta.params[off + n];
        const __half hi = __float2half_rn(bv), lo = __float2half_rn(bv - __half2float(hi));
        uint8_t* tile = base + O_BIAS + 2048 * l;
        *reinterpret_cast<uint4*>(tile + tc::sw32_offset(n, 0)) =
            make_uint4(h2u(__halves2half2(hi, lo)), 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(tile + tc::sw32_offset(n, 1)) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid < 8) {
        const uint32_t ones = h2u(__floats2half2_rn(1.f, 1.f));
        *reinterpret_cast<uint4*>(base + O_ONES + tc::sw32_offset(tid, 0)) =
            make_uint4(ones, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(base + O_ONES + tc::sw32_offset(tid, 1)) =
            make_uint4(0u, 0u, 0u, 0u);
    }
    // dz^T rows 64-127 stay zero; h^T rows 64-79: row 64 all ones, the rest zero
    {
        const uint32_t one2 = h2u(__floats2half2_rn(1.f, 1.f));
        for (int i = tid; i < 2 * 64 * 8; i += TT_THREADS) {
            const int a = i >> 9, r = 64 + ((i >> 3) & 63), c = i & 7;
            *reinterpret_cast<uint4*>(base + O_DT + a * DT_ATOM + tc::sw128_offset(r, c)) =
                make_uint4(0u, 0u, 0u, 0u);
        }
        for (int i = tid; i < 2 * 16 * 8; i += TT_THREADS) {
            const int a = i >> 7, r = 64 + ((i >> 3) & 15), c = i & 7;
            const uint32_t v = r == 64 ? one2 : 0u;
            *reinterpret_cast<uint4*>(base + O_HT + a * HT_ATOM + tc::sw128_offset(r, c)) =
                make_uint4(v, v, v, v);
        }
    }

    // ---- the row's features (normalised, FP16) into x (part 0)
    const int step0 = ta.step ? *ta.step : 0;
    const long long r = (long long)blockIdx.x * 128 + row;
    bool valid;
    long long idx;
    if (ta.sequential) {
        idx = ta.offset + r;
        valid = idx < ta.N;
    } else {
        // lin * perm_mul mod N with both factors reduced mod N first (perm_mul
        // < N from the host, N <= 2^31): the product stays below 2^62 for any
        // step count, so the walk remains a permutation of the rows
        const unsigned long long N = (unsigned long long)ta.N;
        const unsigned long long lin = ((unsigned long long)step0 * (unsigned long long)ta.batch +
                                        (unsigned long long)r) % N;
        idx = (long long)((lin * ta.perm_mul) % N);
        valid = true;
    }
    float tau = -1.f;  // < 0: padding row
    if (part == 0) {
        __align__(16) __half xh[16];
#pragma unroll
        for (int j = 0; j < MLP_IN; ++j) {
            const float f = valid ? ta.feat[(size_t)idx * MLP_IN + j] : 0.f;
            xh[j] = __float2half_rn((f - ta.mu[j]) * ta.inv_sd[j]);
        }
        tau = valid ? ta.tau[idx] : -1.f;
#pragma unroll
        for (int c = 0; c < 2; ++c)
            *reinterpret_cast<uint4*>(base + O_X + tc::sw128_offset(row, c)) =
                *reinterpret_cast<const uint4*>(xh + 8 * c);
    }

    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, TT_COLS);
        tc::tmem_relinquish();
    }
    bool bad = tt_sync(false);
    const uint32_t tmem = *tslot;
    const uint32_t lane_off = (uint32_t)(wq * 32) << 16;
    unsigned phase = 0;
    bool failed = false;
    auto wait = [&]() {
        bad = __any_sync(0xffffffffu, !tc::mbar_wait(bar, phase, ta.wait_ns));
        if (!bad) phase ^= 1u;
        tc::fence_after_sync();
    };

    // ---- forward
    for (int l = 0; l < NL && !failed; ++l) {
        if (tt_sync(bad)) {
            failed = true;
            break;
        }
        if (tid == 0 && !ta.stall) {
            const uint32_t a = sb + (l == 0 ? O_X : (l == 1 ? O_H1 : O_H2));
            if (l == 0)
                tc::mma_f16(tmem, tc::desc_sw128(a), tc::desc_sw32(sb + O_W1), ID64, 0u);
            else
                mma_k(tmem, a, sb + (l == 1 ? O_W2 : O_W3), ID64, 4, 0, 0, false);
            tc::mma_f16(tmem, tc::desc_sw32(sb + O_ONES, 0u), tc::desc_sw32(sb + O_BIAS + 2048u * l),
                        ID64, 1u);
            tc::mma_commit(bar);
        }
        wait();
        if (!bad) {
            float z[CW];
            ld_cols(tmem + lane_off + (uint32_t)c0, z);
            __half* zrow = zs + (size_t)(l * 128 + row) * ZS;
            uint32_t hp[CW / 2];
#pragma unroll
            for (int j = 0; j < CW / 2; ++j) {
                const __half2 zh = __floats2half2_rn(z[2 * j], z[2 * j + 1]);
                *reinterpret_cast<__half2*>(zrow + c0 + 2 * j) = zh;
                const float2 zf = __half22float2(zh);
                hp[j] = h2u(__floats2half2_rn(silu_f(zf.x), silu_f(zf.y)));
            }
            if (l < NL - 1) {
                uint8_t* ht = base + (l == 0 ? O_H1 : O_H2);
#pragma unroll
                for (int c = 0; c < CW / 8; ++c)
                    *reinterpret_cast<uint4*>(ht + tc::sw128_offset(row, c0 / 8 + c)) =
                        make_uint4(hp[4 * c], hp[4 * c + 1], hp[4 * c + 2], hp[4 * c + 3]);
            } else {
                // the part's share of the 64 -> 1 output, summed in part order below
                float yy = 0.f;
#pragma unroll
                for (int j = 0; j < CW / 2; ++j) {
                    const float2 h = __half22float2(*reinterpret_cast<const __half2*>(&hp[j]));
                    yy = fmaf(fw4[c0 + 2 * j], h.x, yy);
                    yy = fmaf(fw4[c0 + 2 * j + 1], h.y, yy);
                }
                fyp[part * 128 + row] = yy;
            }
        }
        tc::fence_before_sync();
    }

    // ---- loss and its gradient (per row, part 0), the output layer's gradients
    __syncthreads();  // the output partials of every part
    float loss = 0.f;
    if (part == 0) {
        float y = ta.params[MLP_B4];
#pragma unroll
        for (int q = 0; q < TT_PARTS; ++q) y += fyp[q * 128 + row];
        float dy = 0.f;
        if (tau >= 0.f) {
            const float k = ta.sigma * ta.tau_scale;
            const float Th = __expf(-k * mlp::softplus(y)), T = __expf(-ta.sigma * tau);
            const float diff = Th - T;
            loss = diff * diff;
            dy = 2.f * diff * (-k * mlp::sigmoid(y) * Th);
        }
        fdy[row] = dy;
    }
    __syncthreads();  // dy of every row
    const float dy = fdy[row];
    {
        // dW4[j] = sum_rows dy h[j] (h: the last hidden layer's activations)
        // and db4 = sum_rows dy: shuffle trees per warp, then the four row
        // groups in order
        const __half* zl = zs + (size_t)((NL - 1) * 128 + row) * ZS;
        for (int j = 0; j < CW; ++j) {
            const float hl = __half2float(__float2half_rn(silu_f(__half2float(zl[c0 + j]))));
            float v = dy * hl;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) fred[wq * 64 + c0 + j] = v;
        }
        if (part == 0) {
            float vb = dy, vl = loss;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                vb += __shfl_xor_sync(0xffffffffu, vb, o);
                vl += __shfl_xor_sync(0xffffffffu, vl, o);
            }
            if (lane == 0) {
                fmisc[wq] = vb;
                fmisc[4 + wq] = vl;
            }
        }
    }

    float* part_out = ta.partial + (size_t)blockIdx.x * (MLP_NPARAM + 1);
    // dz of the layer below from dh (the part's tensor-memory columns) or, for
    // the last hidden layer, from dy w4: FP16 into the dz rows and dz^T
    auto write_dz = [&](int l, const float (&dh)[CW]) {
        const __half* zrow = zs + (size_t)(l * 128 + row) * ZS;
        uint32_t dp[CW / 2];
#pragma unroll
        for (int j = 0; j < CW / 2; ++j) {
            const float2 zf =
                __half22float2(*reinterpret_cast<const __half2*>(zrow + c0 + 2 * j));
            const __half2 d2 = __floats2half2_rn(dh[2 * j] * silu_grad_f(zf.x),
                                                 dh[2 * j + 1] * silu_grad_f(zf.y));
            dp[j] = h2u(d2);
            *reinterpret_cast<__half*>(base + O_DT + kt_addr(c0 + 2 * j, row, DT_ATOM)) =
                __low2half(d2);
            *reinterpret_cast<__half*>(base + O_DT + kt_addr(c0 + 2 * j + 1, row, DT_ATOM)) =
                __high2half(d2);
        }
#pragma unroll
        for (int c = 0; c < CW / 8; ++c)
            *reinterpret_cast<uint4*>(base + O_D + tc::sw128_offset(row, c0 / 8 + c)) =
                make_uint4(dp[4 * c], dp[4 * c + 1], dp[4 * c + 2], dp[4 * c + 3]);
    };
    // h^T (rows 0-63) from a row tile, or x^T (rows 0-15): the part's features
    auto write_ht = [&](const uint8_t* rows, int nfeat) {
        for (int c = c0 / 8; c < (c0 + CW) / 8 && c < nfeat / 8; ++c) {
            const uint4 q = *reinterpret_cast<const uint4*>(rows + tc::sw128_offset(row, c));
            const __half* h = reinterpret_cast<const __half*>(&q);
#pragma unroll
            for (int e = 0; e < 8; ++e)
                *reinterpret_cast<__half*>(base + O_HT + kt_addr(8 * c + e, row, HT_ATOM)) = h[e];
        }
    };
    // rows 0-63 (row groups 0, 1) of tensor-memory cols [64, 160): the part's
    // columns of dW[j][0..nin), and db[j] (part 0)
    auto store_dw = [&](int wo, int bo, int nin) {
        if (wq < 2 && c0 < nin) {
            const int j = row;
            float v[CW];
            ld_cols(tmem + lane_off + 64u + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < CW; ++i) part_out[wo + j * nin + c0 + i] = v[i];
        }
        if (wq < 2 && part == 0) {
            uint32_t rb[16];
            tc::tmem_ld16(tmem + lane_off + 128u, rb);
            part_out[bo + row] = __uint_as_float(rb[0]);
        }
    };

    // the input tile of hidden layer l (x, h1 or h2)
    auto input_of = [&](int l) { return base + (l == 0 ? O_X : (l == 1 ? O_H1 : O_H2)); };
    if (!failed && !bad) {
        // last hidden layer: dz = dy w4 * silu'(z)
        float dh[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) dh[j] = dy * fw4[c0 + j];
        write_dz(NL - 1, dh);
        write_ht(input_of(NL - 1), NL - 1 == 0 ? 16 : 64);
    }
    // backward, from the last hidden layer down: (dW3, dh2), (dW2, dh1), dW1
    for (int l = NL - 1; l >= 0 && !failed; --l) {
        if (tt_sync(bad)) {
            failed = true;
            break;
        }
        if (tid == 0) {
            mma_k(tmem + 64u, sb + O_DT, sb + O_HT, ID80, 8, DT_ATOM, HT_ATOM, false);
            if (l > 0) mma_k(tmem, sb + O_D, sb + (l == 2 ? O_WT3 : O_WT2), ID64, 4, 0, 0, false);
            tc::mma_commit(bar);
        }
        wait();
        float dh[CW];
        if (!bad) {
            store_dw(l == 0 ? MLP_W1 : (l == 1 ? MLP_W2 : MLP_W3),
                     l == 0 ? MLP_B1 : (l == 1 ? MLP_B2 : MLP_B3), l == 0 ? 16 : 64);
            if (l > 0) ld_cols(tmem + lane_off + (uint32_t)c0, dh);
        }
        tc::fence_before_sync();
        if (l > 0) {
            // every warp's tensor-memory loads are done, and the MMAs that read
            // dz, dz^T and h^T have completed, before they are rewritten
            if (tt_sync(bad)) {
                failed = true;
                break;
            }
            write_dz(l - 1, dh);
            write_ht(input_of(l - 1), l - 1 == 0 ? 16 : 64);
            tc::fence_before_sync();
        }
    }
    if (!failed) failed = tt_sync(bad);
    if (failed) {
        // only warps whose wait ran out have a commit pending (no MMA is
        // issued after a failed barrier): drain it, bounded, and agree across
        // the CTA whether every drain completed
        const bool drained = !bad || tc::mbar_wait(bar, phase, ta.wait_ns);
        const bool undrained = __syncthreads_or(!drained) != 0;
        if (tid == 0) {
            part_out[MLP_NPARAM] = __int_as_float(0x7fc00000);  // NaN loss
            // bit 1: tensor memory is freed below with an MMA possibly still
            // in flight, so the host must treat the device as faulted
            atomicOr(ta.status, undrained ? 3ull : 1ull);
        }
    } else {
        if (tid < 64)
            part_out[MLP_W4 + tid] =
                ((fred[tid] + fred[64 + tid]) + fred[128 + tid]) + fred[192 + tid];
        if (tid == 0) {
            part_out[MLP_B4] = ((fmisc[0] + fmisc[1]) + fmisc[2]) + fmisc[3];
            part_out[MLP_NPARAM] = ((fmisc[4] + fmisc[5]) + fmisc[6]) + fmisc[7];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TT_COLS);
    if (ta.grid_bar) fused_adam(ta, step0, reinterpret_cast<int*>(fmisc + 8));
}

using TrainFn = void (*)(TrainArgs);
const TrainFn kTrainFns[MLP_MAX_LAYERS] = {k_mlp_train_tc<1>, k_mlp_train_tc<2>,
                                           k_mlp_train_tc<3>};

}  // namespace

// CTAs of the training kernel resident at once on the current device (set
// up once per device, outside any stream capture; 0 on an error).
int mlp_train_resident_ctas() {
    static std::atomic<int> resident[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int r = resident[dev].load(std::memory_order_acquire);
    if (r > 0) return r;
    for (TrainFn fn : kTrainFns)
        if (cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TT_SMEM) != cudaSuccess)
            return 0;
    // the fewest resident CTAs over the depths (they share the shared-memory
    // layout and the launch bounds)
    int per_sm = 1 << 30, sms = 0;
    for (TrainFn fn : kTrainFns) {
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, (const void*)fn, TT_THREADS, TT_SMEM) !=
            cudaSuccess)
            return 0;
        per_sm = std::min(per_sm, k);
    }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    r = per_sm * sms;
    resident[dev].store(r, std::memory_order_release);
    return r;
}

cudaError_t launch_mlp_train(const TrainArgs& ta, int ctas, cudaStream_t st) {
    if (ta.layers < 1 || ta.layers > MLP_MAX_LAYERS) return cudaErrorInvalidValue;
    const TrainFn fn = kTrainFns[ta.layers - 1];
    const int resident = mlp_train_resident_ctas();
    if (resident <= 0) return cudaErrorInvalidConfiguration;
    if (!ta.grid_bar) {
        fn<<<ctas, TT_THREADS, TT_SMEM, st>>>(ta);
        return cudaGetLastError();
    }
    // the fused optimiser's grid barrier needs every CTA resident: a
    // cooperative launch, refused when the grid does not fit
    if (ctas > resident) return cudaErrorCooperativeLaunchTooLarge;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(TT_THREADS);
    cfg.dynamicSmemBytes = TT_SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fn, ta);
}

CG_OOB_TU(k_train_tc)
