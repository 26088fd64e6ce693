// k_shade_tc.cu -- the surrogate's inference on the fifth-generation tensor
// cores: sun transmittance of every recorded view sample through the MLP
// (16 -> NL x 64 SiLU -> 1 with NL = 1, 2 or 3 hidden layers, a template
// parameter; FP16 operands, FP32 accumulation).
//
// One CTA = 4 warps (thread = row of a 128-row tile), persistent over tiles.
// Per tile:
//   1. each thread's row holds the normalised FP16 features of its sample in
//      the activation tile (shared memory, 128B-swizzled K-major);
//   2. thread 0 issues layer 1 (one tcgen05.mma, M=128 N=64 K=16) into tensor
//      memory and commits it to an mbarrier;
//   3. each warp reads its 32 rows back (tcgen05.ld), applies SiLU and writes
//      the next activation tile in place as FP16; hidden layers 2 and 3 are 4
//      MMAs each (K = 64); every layer ends with one more K = 16 MMA that adds
//      the bias (a column of ones against the bias split into two FP16 halves);
//   4. the last epilogue folds the 64 -> 1 output layer into FP32 FMAs, then
//      the softplus link, the transmittance and the sample's contribution;
//      the next tile's inputs go into the tile.
// The next tile is fetched in stages while this one runs, so that no load is
// consumed in the phase that issued it: its slot (during the tile before),
// its sample (layer 1), its 12 texture taps (the last layer), its inputs
// (output); with one layer slot, sample and taps share the one phase.  Tiles are
// claimed dynamically (an atomic counter, two tiles ahead of the one being
// shaded): CTAs on slower SMs (the far die's L2, texture misses) take fewer
// tiles instead of setting the kernel's tail.
// Hidden layers run on weights and biases pre-scaled by 1/2 (exact in FP16
// and FP32), so the accumulator holds z/2 and SiLU is z/2 * (1 + tanh(z/2)).
// Every mbarrier wait is bounded (1 s of the global timer): on a timeout the
// CTA records an error, waits (bounded) for its MMA to drain, frees its tensor
// memory and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>

#include "cg_internal.h"
#include "cg_mlp.cuh"
#include "cg_mlp_tc.cuh"
#include "cg_sample.cuh"
#include "cg_tc.cuh"

namespace {

constexpr uint32_t TC_TMEM_COLS = 64;
constexpr uint64_t TC_WAIT_NS = 1000000000ull;  // 1 s: a wait longer than this is a fault
// CTAs per SM by depth: the register budget (__launch_bounds__) and the
// shared memory (the network tiles of the model's layers) allow five for
// three hidden layers and SHALLOW_CTAS_PER_SM for fewer
constexpr int SHALLOW_CTAS_PER_SM = 6;
template <int NL>
constexpr int ctas_per_sm() { return NL >= 3 ? 5 : SHALLOW_CTAS_PER_SM; }
// shared memory map of k_mlp_infer_tc (bytes from the 1024-aligned base)
constexpr int OFF_ACT = 0;      // 128 x 128 B activation tile (SW128)
constexpr int OFF_NET = 16384;  // the network tiles (cg_mlp_tc.cuh)
template <int NL>
struct InferSmem {
    static constexpr int OFF_BAR = OFF_NET + mlptc::Net<NL>::BYTES;  // mbarrier + TMEM address
    static constexpr int BYTES = OFF_BAR + 32 + 1024;                // + alignment slack
    static_assert((BYTES + 1024) * ctas_per_sm<NL>() <= 228 * 1024, "infer shared memory");
};

// The exact cone for a sample whose features left the trained range (rare):
// kept out of line so that the hot loop's registers are not sized for it.
template <int FMT>
__device__ __noinline__ float exact_tau(const VolDesc& vd, const ConeSchedule& cone, float x,
                                        float y, float z, const float* sun) {
    return cgs::sun_cone<FMT>(vd, cone, x, y, z, sun[0], sun[1], sun[2]);
}

// A tile row in flight: its sample slot, the output's inputs (weight, light)
// and the exact-cone optical depth when a feature fell outside the trained
// range (tau_fb >= 0), computed when the features were.
struct Row {
    unsigned slot;
    float w, g, tau_fb;
};

// The 12 texture taps and the other inputs of a sample (issued early; the
// results are consumed by pack_row).
__device__ __forceinline__ void fetch_features(const FeatGeom& geo, const TraceParams& tp,
                                               unsigned slot, const float4& s,
                                               float (&f)[MLP_IN]) {
    if (slot != CG_NO_SLOT) {
        mlp::features(geo, s.x, s.y, s.z, tp.sun[0], tp.sun[1], tp.sun[2], f);
    } else {
#pragma unroll
        for (int j = 0; j < MLP_IN; ++j) f[j] = 0.f;
    }
}

// Features -> the row state and the normalised FP16 inputs in chunks 0-1 of
// the thread's tile row.
template <int FMT>
__device__ __forceinline__ void pack_row(const VolDesc& vd, const ConeSchedule& cone,
                                         const MlpDev& m, const TraceParams& tp, unsigned slot,
                                         const float4& s, float g, const float (&f)[MLP_IN],
                                         Row& r, uint8_t* act, int row) {
    r.slot = slot;
    r.w = s.w;
    r.g = g;
    r.tau_fb = -1.f;
    if (slot != CG_NO_SLOT && !mlp::in_range(m, f))
        r.tau_fb = exact_tau<FMT>(vd, cone, s.x, s.y, s.z, tp.sun);
    mlptc::write_inputs(act, row, m, f, slot != CG_NO_SLOT);
}

__device__ __forceinline__ unsigned slot_at(const SampleBuf& sb, unsigned tile, unsigned ntiles,
                                            unsigned total, int row) {
    const unsigned i = tile * 128u + (unsigned)row;
    const unsigned s = (tile < ntiles && i < total) ? sb.slot_of[i] : CG_NO_SLOT;
    return (s == CG_NO_SLOT || CG_IN_BOUNDS(s, sb.nslots)) ? s : CG_NO_SLOT;
}

// All writes of the CTA to the activation tiles -> visible to the tensor
// core, then one thread issues.  The same barrier agrees on a failed wait of
// any thread (true: the CTA stops before issuing).
__device__ __forceinline__ bool sync_for_mma(bool bad) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    const bool any_bad = __syncthreads_or(bad) != 0;
    tc::fence_after_sync();
    return any_bad;
}

// After a failed barrier (CTA-uniform): drain the outstanding commit, bounded
// (only warps whose wait ran out have one: no MMA is issued after a failed
// barrier), agree across the CTA whether every drain completed, and report:
// status[1] |= 1, and |= 2 when a drain ran out too (tensor memory is then
// freed with an MMA possibly in flight: the host treats the device as faulted).
__device__ __forceinline__ void report_failure(uint64_t* bar, unsigned phase, bool bad,
                                               unsigned long long* status) {
    const bool drained = !bad || tc::mbar_wait(bar, phase, TC_WAIT_NS);
    const bool undrained = __syncthreads_or(!drained) != 0;
    if (threadIdx.x == 0) atomicOr(status + 1, undrained ? 3ull : 1ull);
}

// ---- the shade kernel: SHADE_GROUPS independent 4-warp groups per CTA, each
// with its own activation tile, tensor-memory columns, mbarrier and tile
// stream, sharing one copy of the network tiles (so that more groups fit an
// SM's shared memory than CTAs of one group would).
constexpr int SHADE_GROUPS = 1;
constexpr uint32_t SHADE_TMEM_COLS = SHADE_GROUPS == 1 ? 64u : (SHADE_GROUPS == 2 ? 128u : 256u);
constexpr int SH_OFF_NET = SHADE_GROUPS * mlptc::ACT_BYTES;
template <int NL>
struct ShadeSmem {
    static constexpr int OFF_BAR = SH_OFF_NET + mlptc::Net<NL>::BYTES;  // bar[G], tmem slot, claim[G]
    static constexpr int BYTES = OFF_BAR + 8 * SHADE_GROUPS + 4 + 4 * SHADE_GROUPS + 1024;
    static_assert((BYTES + 1024) * ctas_per_sm<NL>() <= 228 * 1024, "shade shared memory");
    static_assert(SHADE_TMEM_COLS * ctas_per_sm<NL>() <= 512, "tensor memory");
};

// The group's barrier (named barrier 1 + g, 128 threads) that also agrees on
// a failed wait of any of its threads.
__device__ __forceinline__ bool group_sync_or(int g, bool v) {
    if (SHADE_GROUPS == 1) return __syncthreads_or(v) != 0;
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n"
        " bar.red.or.pred p, %2, 128, q;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + g)
        : "memory");
    return r != 0;
}

// All writes of the group to its activation tile -> visible to the tensor
// core, then its first thread issues; true when a wait of the group ran out.
__device__ __forceinline__ bool group_sync_for_mma(int g, bool bad) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    const bool any_bad = group_sync_or(g, bad);
    tc::fence_after_sync();
    return any_bad;
}

template <int FMT, int NL>
__global__ void __launch_bounds__(128 * SHADE_GROUPS, ctas_per_sm<NL>())
    k_shade_mlp_tc(const __grid_constant__ VolDesc vd, const __grid_constant__ TraceParams tp,
                   const __grid_constant__ ConeSchedule cone, const __grid_constant__ MlpDev m,
                   const __grid_constant__ FeatGeom geo, SampleBuf sb,
                   unsigned long long* status) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_addr(smem_raw);
    uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = tid >> 7, r = tid & 127;  // group, row of the group's tile
    uint8_t* act = base + g * mlptc::ACT_BYTES;
    constexpr int OB = ShadeSmem<NL>::OFF_BAR;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + OB) + g;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + OB + 8 * SHADE_GROUPS);
    unsigned* s_claim = reinterpret_cast<unsigned*>(base + OB + 8 * SHADE_GROUPS + 4) + g;

    mlptc::stage_network<NL>(base + SH_OFF_NET, m, tid, blockDim.x);
    if (r == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, SHADE_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    grid_dep_wait();  // the march's samples and flat order
    const uint32_t tmem = *tslot + 64u * (uint32_t)g;
    const uint32_t dw = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t a_addr = tc::smem_addr(act);
    const uint32_t net_addr = tc::smem_addr(base + SH_OFF_NET);
    const float amb = tp.ambient;
    const unsigned total = *sb.flat_total;
    const unsigned ntiles = (total + 127u) / 128u;
    const unsigned streams = gridDim.x * SHADE_GROUPS;
    unsigned phase = 0, n_fallback = 0, n_valid = 0;
    bool failed = false, bad = false;  // bad: a wait of this warp ran out

    // ---- the first tile's inputs
    unsigned tile = blockIdx.x * SHADE_GROUPS + g;
    Row row;
    {
        const unsigned slot = slot_at(sb, tile, ntiles, total, r);
        float4 sp = make_float4(0.f, 0.f, 0.f, 0.f);
        float gl = 0.f;
        if (slot != CG_NO_SLOT) {
            sp = sb.pos_w[slot];
            gl = sb.light_lane[slot].x;
        }
        float f[MLP_IN];
        fetch_features(geo, tp, slot, sp, f);
        pack_row<FMT>(vd, cone, m, tp, slot, sp, gl, f, row, act, r);
    }

    // the first two tiles of a group are static, later ones are claimed from
    // status[3]
    unsigned ntile = tile + streams;
    // with two or more layers a tile's slot is fetched one tile ahead (at
    // layer 1 of the tile before, from the claim made at its layer 0)
    unsigned nslot = NL >= 2 ? slot_at(sb, ntile, ntiles, total, r) : CG_NO_SLOT;
    for (; tile < ntiles;) {
        unsigned nnslot = CG_NO_SLOT, nntile = 0u;
        float4 ns = make_float4(0.f, 0.f, 0.f, 0.f);
        float ng = 0.f;
        float nf[MLP_IN];
        float y = 0.f;
#pragma unroll
        for (int layer = 0; layer < NL; ++layer) {
            if (group_sync_for_mma(g, bad)) {  // a commit of parity `phase` is still pending
                failed = true;
                break;
            }
            if (r == 0) {
                mlptc::issue_layer<NL>(layer, tmem, a_addr, net_addr, bar);
                // claim the tile after next (read by the group after the next sync)
                if (layer == 0) *s_claim = 2u * streams + (unsigned)atomicAdd(status + 3, 1ull);
            }
            // ---- the next tile, in stages: its sample (layer 0), the slot of
            // the tile after it (layer 1), its texture taps (last layer); one
            // layer: slot, sample and taps in the same phase
            if (NL == 1) nslot = slot_at(sb, ntile, ntiles, total, r);
            if (layer == 0 && nslot != CG_NO_SLOT) {
                ns = sb.pos_w[nslot];
                ng = sb.light_lane[nslot].x;
            }
            if (NL >= 2 && layer == 1) {
                nntile = *s_claim;  // written at layer 0, one barrier ago
                nnslot = slot_at(sb, nntile, ntiles, total, r);
            }
            if (layer == NL - 1) fetch_features(geo, tp, nslot, ns, nf);
            // a warp whose wait ran out skips the epilogue (no tensor-memory
            // read under a running MMA) and the group stops at the next barrier
            bad = __any_sync(0xffffffffu, !tc::mbar_wait(bar, phase, TC_WAIT_NS));
            if (!bad) phase ^= 1u;
            tc::fence_after_sync();
            // ---- epilogue: TMEM -> bias + SiLU, 32 columns at a time; the
            // last layer folds the 64 -> 1 output in FP32
            if (!bad) {
                const float yy = mlptc::layer_epilogue(layer == NL - 1, dw, act, r, m);
                if (layer == NL - 1) y = yy;
            }
            tc::fence_before_sync();
        }
        if (failed) break;
        // ---- output
        if (row.slot != CG_NO_SLOT && !bad) {
            n_valid++;
            float tau;
            if (row.tau_fb >= 0.f) {
                tau = row.tau_fb;
                n_fallback++;
            } else {
                tau = m.tau_scale * mlp::softplus(y);
            }
            if (CG_IN_BOUNDS(row.slot, sb.nslots))
                sb.contrib[row.slot] =
                    row.w * __expf(-tp.sigma * tau) * (amb + (1.f - amb) * row.g);
        }
        // ---- the next tile's inputs
        pack_row<FMT>(vd, cone, m, tp, nslot, ns, ng, nf, row, act, r);
        tile = ntile;
        if (NL >= 2) {
            ntile = nntile;
            nslot = nnslot;
        } else {
            ntile = *s_claim;  // written at layer 0, one barrier ago
        }
    }
    if (!failed) failed = group_sync_for_mma(g, bad);  // the last tile's waits
    if (failed) {
        // drain the outstanding commit (bounded; only warps whose wait ran
        // out have one), agree within the group whether every drain
        // completed, and report (|= 2: tensor memory is freed below with an
        // MMA possibly in flight; the host treats the device as faulted)
        const bool drained = !bad || tc::mbar_wait(bar, phase, TC_WAIT_NS);
        const bool undrained = group_sync_or(g, !drained);
        if (r == 0) atomicOr(status + 1, undrained ? 3ull : 1ull);
    }
    unsigned tot = n_fallback, nv = n_valid;
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        nv += __shfl_xor_sync(0xffffffffu, nv, o);
    }
    if (lane == 0) {
        if (tot) atomicAdd(status, (unsigned long long)tot);
        if (nv) atomicAdd(status + 2, (unsigned long long)nv);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(*tslot, SHADE_TMEM_COLS);
}

// The network alone over n rows of raw features (normalised here):
// out[i] = tau_scale * softplus(y_i).  The tile pipeline of k_shade_mlp_tc
// without the sample fetches: 128-row tiles at a static stride, the same
// staged weights, layers, epilogues and bounded waits.
template <int NL>
__global__ void __launch_bounds__(128, ctas_per_sm<NL>())
    k_mlp_infer_tc(const __grid_constant__ MlpDev m, const float* feat, int n, float* out,
                   unsigned long long* status) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_addr(smem_raw);
    uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* act = base + OFF_ACT;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + InferSmem<NL>::OFF_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + InferSmem<NL>::OFF_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    mlptc::stage_network<NL>(base + OFF_NET, m, tid, blockDim.x);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, TC_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t dw = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t a_addr = tc::smem_addr(act);
    const uint32_t net_addr = tc::smem_addr(base + OFF_NET);
    unsigned phase = 0;
    bool failed = false, bad = false;  // bad: a wait of this warp ran out
    const int ntiles = (n + 127) / 128;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row = tile * 128 + tid;
        // this row's normalised FP16 features into chunks 0-1 of its tile row
        // (the previous tile's last MMA, the last reader, has completed)
        uint32_t x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float f0 = row < n ? feat[(size_t)row * MLP_IN + 2 * q] : m.mu[2 * q];
            const float f1 = row < n ? feat[(size_t)row * MLP_IN + 2 * q + 1] : m.mu[2 * q + 1];
            x[q] = mlp::pack_h2((f0 - m.mu[2 * q]) * m.inv_sd[2 * q],
                                (f1 - m.mu[2 * q + 1]) * m.inv_sd[2 * q + 1]);
        }
        *reinterpret_cast<uint4*>(act + tc::sw128_offset(tid, 0)) =
            make_uint4(x[0], x[1], x[2], x[3]);
        *reinterpret_cast<uint4*>(act + tc::sw128_offset(tid, 1)) =
            make_uint4(x[4], x[5], x[6], x[7]);
        float y = 0.f;
#pragma unroll
        for (int layer = 0; layer < NL; ++layer) {
            if (sync_for_mma(bad)) {  // a commit of parity `phase` is still pending
                failed = true;
                break;
            }
            if (tid == 0)
                mlptc::issue_layer<NL>(layer, tmem, a_addr, net_addr, bar);
            bad = __any_sync(0xffffffffu, !tc::mbar_wait(bar, phase, TC_WAIT_NS));
            if (!bad) phase ^= 1u;
            tc::fence_after_sync();
            if (!bad) {
                const float yy = mlptc::layer_epilogue(layer == NL - 1, dw, act, tid, m);
                if (layer == NL - 1) y = yy;
            }
            tc::fence_before_sync();
        }
        if (failed) break;
        if (row < n && !bad) out[row] = m.tau_scale * mlp::softplus(y);
    }
    if (!failed) failed = sync_for_mma(bad);  // the last tile's waits
    if (failed) report_failure(bar, phase, bad, status);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

// The bounded wait on an mbarrier that nothing arrives on: one CTA inits the
// barrier, waits for its first phase with the time limit, and records the
// outcome in the status block ([1] |= 1 on a timeout, [3] = nanoseconds
// waited); the kernel then returns normally.
__global__ void k_wait_probe(uint64_t limit_ns, unsigned long long* status) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    const uint64_t t0 = tc::global_ns();
    const bool ok = tc::mbar_wait(&bar, 0u, limit_ns);
    const uint64_t dt = tc::global_ns() - t0;
    if (__syncthreads_or(!ok) && threadIdx.x == 0) {
        atomicOr(status + 1, 1ull);
        status[3] = dt;
    }
}

}  // namespace

cudaError_t launch_wait_probe(uint64_t limit_ns, unsigned long long* status, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(limit_ns, status);
    return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const MlpDev& m, const float* feat, int n, float* out,
                             unsigned long long* status, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (m.layers < 1 || m.layers > MLP_MAX_LAYERS) return cudaErrorInvalidValue;
    // the shared-memory attributes and the SM count are set up once per device
    static std::atomic<int> sm_count[64];
    using InferFn = void (*)(MlpDev, const float*, int, float*, unsigned long long*);
    const InferFn fns[MLP_MAX_LAYERS] = {k_mlp_infer_tc<1>, k_mlp_infer_tc<2>, k_mlp_infer_tc<3>};
    const int smem[MLP_MAX_LAYERS] = {InferSmem<1>::BYTES, InferSmem<2>::BYTES,
                                      InferSmem<3>::BYTES};
    const int per_sm[MLP_MAX_LAYERS] = {ctas_per_sm<1>(), ctas_per_sm<2>(), ctas_per_sm<3>()};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!sm_count[dev].load(std::memory_order_acquire)) {
        for (int i = 0; i < MLP_MAX_LAYERS; ++i) {
            e = cudaFuncSetAttribute((const void*)fns[i],
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem[i]);
            if (e != cudaSuccess) return e;
        }
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        sm_count[dev].store(sms, std::memory_order_release);
    }
    const int L = m.layers - 1;
    const int ntiles = (n + 127) / 128;
    const int blocks = std::min(sm_count[dev].load(std::memory_order_acquire) * per_sm[L], ntiles);
    fns[L]<<<blocks, 128, smem[L], st>>>(m, feat, n, out, status);
    return cudaGetLastError();
}

cudaError_t launch_shade_mlp_tc(VolDesc vd, CamDesc cam, TraceParams tp, const MlpDev& m,
                                SampleBuf sb, unsigned long long* status, cudaStream_t st) {
    (void)cam;
    ConeSchedule cone = make_cone_schedule(vd, tp);
    const FeatGeom geo = feat_geom(vd, m);
    // (the shared-memory attributes and the SM count are configured once per
    // device; atomics keep concurrent host threads well-defined)
    if (m.layers < 1 || m.layers > MLP_MAX_LAYERS) return cudaErrorInvalidValue;
    static std::atomic<int> sm_count[64];
    using ShadeFn = void (*)(VolDesc, TraceParams, ConeSchedule, MlpDev, FeatGeom, SampleBuf,
                             unsigned long long*);
    const ShadeFn fns[2][MLP_MAX_LAYERS] = {
        {k_shade_mlp_tc<0, 1>, k_shade_mlp_tc<0, 2>, k_shade_mlp_tc<0, 3>},
        {k_shade_mlp_tc<1, 1>, k_shade_mlp_tc<1, 2>, k_shade_mlp_tc<1, 3>}};
    const int smem[MLP_MAX_LAYERS] = {ShadeSmem<1>::BYTES, ShadeSmem<2>::BYTES,
                                      ShadeSmem<3>::BYTES};
    const int per_sm[MLP_MAX_LAYERS] = {ctas_per_sm<1>(), ctas_per_sm<2>(), ctas_per_sm<3>()};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!sm_count[dev].load(std::memory_order_acquire)) {
        for (int f = 0; f < 2; ++f)
            for (int i = 0; i < MLP_MAX_LAYERS; ++i) {
                e = cudaFuncSetAttribute((const void*)fns[f][i],
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem[i]);
                if (e != cudaSuccess) return e;
            }
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        sm_count[dev].store(sms, std::memory_order_release);
    }
    // one persistent wave: ctas_per_sm<NL>() CTAs per SM (64 tensor-memory
    // columns each)
    const int L = m.layers - 1;
    const int blocks = sm_count[dev].load(std::memory_order_acquire) * per_sm[L];
    // launched as a dependent of the march: the prologue (network tiles,
    // barrier, tensor memory) overlaps the march's last wave
    return launch_dependent(fns[vd.fmt == 0 ? 0 : 1][L], dim3(blocks), dim3(128 * SHADE_GROUPS),
                            (size_t)smem[L], st, vd, tp, cone, m, geo, sb, status);
}

CG_OOB_TU(k_shade_tc)
