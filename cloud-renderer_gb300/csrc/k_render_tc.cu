// k_render_tc.cu -- the surrogate renderer as one persistent, warp-specialised
// kernel: view march -> sun-transmittance MLP on the tensor cores ->
// front-to-back composite, with no sample records in global memory between
// the stages (the deferred form, k_march -> k_shade_mlp_tc -> k_accumulate,
// writes 24-byte records of every contributing sample and reads them back).
//
// Work unit: a region = one 8x4-pixel tile of the image (one ray per lane),
// regions numbered in raster order and claimed dynamically.  Per CTA (three
// per SM, 256 threads; the fastest of the shapes measured):
//   warps 0-3   epilogue: one thread per row of a 128-sample tile; features
//               (12 texture taps), FP16 inputs into the activation tile, the
//               SiLU epilogues of the hidden layers (tensor memory -> FP16
//               activations in place), the 64 -> 1 output, the sample's
//               contribution w * exp(-sigma tau) * (ambient + (1 - ambient) G)
//               into the region's contribution slots;
//   warp 4      the tensor-core issuer: per tile and layer, waits until the
//               epilogue has written the activations, issues the layer's
//               tcgen05.mma (M = 128, N = 64, FP16 operands, FP32 tensor-memory
//               accumulators) and commits it to an mbarrier;
//   warps 5-7   producers: march their region with k_march's texture-filtered
//               march (cg_march.cuh: same samples, same (step, lane) order), append every
//               contributing sample (voxel position, weight T*alpha, light G,
//               record and slot) to a ring of RT_RING 128-row staging tiles in
//               shared memory, record the region's step table, and once all of
//               a region's samples are shaded, composite its 32 pixels in step
//               order (Neumaier) -- the order of k_accumulate, so images equal
//               the deferred form's.
// Synchronisation: staging tile t lives in ring slot t % RT_RING; producers
// claim rows with a shared counter, wait until the slot's previous tile has
// been read (a shared counter of released tiles), write the rows and arrive on
// the slot's mbarrier (128 arrivals per tile).  A producer about to wait for
// one of its regions pads that region's last tile (empty rows) if it is not
// yet full, so that no wait depends on rows nobody will write.  The last
// producer to finish marks the end with a tile whose number the epilogue
// recognises; the epilogue then tells the issuer to stop.  Every wait is
// bounded (1 s of the global timer): on a timeout the CTA sets an abort flag,
// every role leaves its loop, the issuer drains its last commit (bounded) and
// the status word reports the failure.
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "cg_internal.h"
#include "cg_march.cuh"
#include "cg_mlp.cuh"
#include "cg_mlp_tc.cuh"
#include "cg_sample.cuh"
#include "cg_tc.cuh"

namespace {

constexpr int RT_EPI_WARPS = 4;
constexpr int RT_MMA_WARP = 4;
constexpr int RT_PRODUCERS = 3;
constexpr int RT_FIRST_PRODUCER = RT_EPI_WARPS + 1;
constexpr int RT_THREADS = 32 * (RT_EPI_WARPS + 1 + RT_PRODUCERS);
constexpr int RT_CTAS_PER_SM = 3;
constexpr int RT_RING = 8;    // staging tiles of 128 rows
constexpr int RT_RECS = 4;    // region records per producer warp
constexpr uint32_t RT_TMEM_COLS = 64;
constexpr uint64_t RT_WAIT_NS = 1000000000ull;  // 1 s: a wait longer than this is a fault
constexpr unsigned RT_NO_REC = 0xFFFFu;          // meta of an empty row
constexpr unsigned RT_IN_PROGRESS = 0xFFFFFFFFu;

// A region in flight: written by its producer, `done` counted up by the
// epilogue as the region's samples are shaded.
struct Rec {
    unsigned region;
    unsigned count;     // samples (RT_IN_PROGRESS while the march runs)
    unsigned done;      // samples shaded
    unsigned nsteps;    // emitting steps (entries of the step table)
    unsigned last_row;  // staging row of the last sample
    unsigned busy;      // 1 until composited
    unsigned pad[2];
    float T[32];        // per lane: the ray's final transmittance
};

// shared memory map (bytes from the 1024-aligned base)
constexpr int OFF_ACT = 0;
constexpr int OFF_NET = OFF_ACT + mlptc::ACT_BYTES;
// the three-layer network layout (a model of any depth runs in it)
using RtNet = mlptc::Net<MLP_MAX_LAYERS>;
constexpr int OFF_POS = OFF_NET + RtNet::BYTES;              // float4 [RING * 128]
constexpr int OFF_META = OFF_POS + RT_RING * 128 * 16;        // uint2 [RING * 128]
constexpr int OFF_REC = OFF_META + RT_RING * 128 * 8;         // Rec [PRODUCERS][RECS]
constexpr int OFF_BAR = OFF_REC + RT_PRODUCERS * RT_RECS * (int)sizeof(Rec);
// barriers: full[RING], act_ready, mma_done; then the shared words
constexpr int OFF_WORDS = OFF_BAR + 8 * (RT_RING + 2);
constexpr int W_TMEM = 0, W_TAIL = 1, W_RELEASED = 2, W_PDONE = 3, W_END = 4, W_ABORT = 5,
              W_STOP = 6, W_COUNT = 8;
constexpr int RT_SMEM_USED = OFF_WORDS + 4 * W_COUNT;
constexpr int RT_SMEM_BYTES = RT_SMEM_USED + 1024;
static_assert(OFF_NET % 1024 == 0 && OFF_POS % 16 == 0 && OFF_BAR % 8 == 0, "alignment");
static_assert(RT_SMEM_BYTES * RT_CTAS_PER_SM <= 227 * 1024, "shared memory");

struct Shared {
    uint8_t* act;
    uint8_t* net;
    float4* pos;
    uint2* meta;
    Rec* rec;
    uint64_t* full;
    uint64_t* act_ready;
    uint64_t* mma_done;
    unsigned* w;
};

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
    return *reinterpret_cast<const volatile unsigned*>(p);
}
__device__ __forceinline__ void st_volatile(unsigned* p, unsigned v) {
    *reinterpret_cast<volatile unsigned*>(p) = v;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     tc::smem_addr(bar)),
                 "r"(count)
                 : "memory");
}

// The epilogue warps' own barrier (named barrier 1, 128 threads): a plain
// sync, and a sync that returns whether any of the 128 threads passed true.
__device__ __forceinline__ void epi_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(RT_EPI_WARPS * 32) : "memory");
}
__device__ __forceinline__ bool epi_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n"
        " bar.red.or.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(RT_EPI_WARPS * 32)
        : "memory");
    return r != 0;
}

// Record an abort: every role leaves its loop at its next wait.
__device__ __forceinline__ void abort_cta(const Shared& S, unsigned long long* status) {
    st_volatile(S.w + W_ABORT, 1u);
    atomicOr(status + 1, 1ull);
}

// Wait for the phase with parity `phase` of `bar`, bounded by the global
// timer and cut short by an abort; false when the CTA is aborting.
__device__ __forceinline__ bool wait_phase(const Shared& S, uint64_t* bar, unsigned phase,
                                           unsigned long long* status) {
    if (tc::mbar_try_wait(bar, phase)) return true;
    const uint64_t t0 = tc::global_ns();
    while (!tc::mbar_try_wait(bar, phase)) {
        if (ld_volatile(S.w + W_ABORT)) return false;
        if (tc::global_ns() - t0 > RT_WAIT_NS) {
            abort_cta(S, status);
            return false;
        }
    }
    return true;
}

// Spin (one lane) until `pred()` holds, bounded; false when aborting.
template <class P>
__device__ __forceinline__ bool spin_until(const Shared& S, P pred, unsigned long long* status) {
    if (pred()) return true;
    const uint64_t t0 = tc::global_ns();
    while (!pred()) {
        if (ld_volatile(S.w + W_ABORT)) return false;
        if (tc::global_ns() - t0 > RT_WAIT_NS) {
            abort_cta(S, status);
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

// ---- producers ---------------------------------------------------------------

struct RenderArgs {
    float* contrib;   // per region: 32 * view_steps contribution slots
    uint2* steps;     // per region: view_steps (first slot, lane ballot) entries
    float4* dst;      // finished pixels (device image or device-addressable host image)
    int regions, tiles_x, cap;
};

// Claim rows [old, end) of the ring up to the end of the tile holding `row`
// (so that the tile completes) and publish them as empty rows.  One warp.
__device__ bool pad_tile(const Shared& S, unsigned row, unsigned long long* status) {
    const int lane = threadIdx.x & 31;
    const unsigned end = (row / 128u + 1u) * 128u;
    unsigned old = 0;
    if (lane == 0) {
        old = ld_volatile(S.w + W_TAIL);
        while (old < end) {
            const unsigned got = atomicCAS(S.w + W_TAIL, old, end);
            if (got == old) break;
            old = got;
        }
    }
    old = __shfl_sync(0xffffffffu, old, 0);
    if (old >= end) return true;  // someone else's rows complete the tile
    const unsigned t = old / 128u;
    bool ok = true;
    if (lane == 0)
        ok = spin_until(S, [&] { return ld_volatile(S.w + W_RELEASED) + RT_RING > t; }, status);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) return false;
    unsigned mine = 0;
    for (unsigned r = old + lane; r < end; r += 32u) {
        S.meta[r % (RT_RING * 128u)] = make_uint2(0u, RT_NO_REC << 16);
        mine++;
    }
    if (mine) mbar_arrive(S.full + t % RT_RING, mine);
    return true;
}

// Wait until every sample of record `rc` is shaded, then write its 32 pixels:
// each lane sums its own samples' contributions in step order (Neumaier).
__device__ bool finish_region(const Shared& S, Rec& rc, const RenderArgs& ra,
                              const CamDesc& cam, const TraceParams& tp, int view_steps,
                              unsigned long long* status) {
    const int lane = threadIdx.x & 31;
    const unsigned n = rc.count;
    if (n > 0) {
        // the region's last tile must be able to complete
        if (!pad_tile(S, rc.last_row, status)) return false;
        bool ok = true;
        if (lane == 0) ok = spin_until(S, [&] { return ld_volatile(&rc.done) >= n; }, status);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) return false;
        __threadfence_block();  // the epilogue's contribution stores before its count
    }
    const unsigned below = (1u << lane) - 1u;
    const unsigned ns = rc.nsteps;
    const uint2* steps = ra.steps + (size_t)rc.region * view_steps;
    const float* cw = ra.contrib + (size_t)rc.region * ra.cap;
    float acc = 0.f, comp = 0.f;
    for (unsigned base = 0; base < ns; base += 32u) {
        const unsigned m = min(32u, ns - base);
        const uint2 st_l = lane < (int)m ? steps[base + lane] : make_uint2(0u, 0u);
        for (unsigned e0 = 0; e0 < m; e0 += 8u) {
            float v[8];
            unsigned have = 0u;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int src = (int)(e0 + q) & 31;
                const unsigned sx = __shfl_sync(0xffffffffu, st_l.x, src);
                const unsigned sy = __shfl_sync(0xffffffffu, st_l.y, src);
                v[q] = 0.f;
                if (e0 + q < m && ((sy >> lane) & 1u)) {
                    v[q] = cw[sx + __popc(sy & below)];
                    have |= 1u << q;
                }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if ((have >> q) & 1u) cgs::neumaier(acc, comp, v[q]);
        }
    }
    const int px = (int)(rc.region % (unsigned)ra.tiles_x) * 8 + (lane & 7);
    const int py = (int)(rc.region / (unsigned)ra.tiles_x) * 4 + (lane >> 3);
    if (px < cam.W && py < cam.H) {
        const float C = acc + comp;
        ra.dst[(size_t)py * cam.W + px] =
            make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2],
                        1.f - rc.T[lane]);
    }
    __syncwarp();
    if (lane == 0) rc.busy = 0u;
    __syncwarp();
    return true;
}

// March region `region` (cg_march.cuh: the samples and order of k_march's
// texture-filtered form), appending every contributing sample to the staging
// ring; fills record `rc` (index `ri`).
__device__ bool march_region(const Shared& S, Rec& rc, unsigned ri, unsigned region,
                             const VolDesc& vd, const CamDesc& cam, const TraceParams& tp,
                             const RenderArgs& ra, unsigned long long* status) {
    const int lane = threadIdx.x & 31;
    const int px = (int)(region % (unsigned)ra.tiles_x) * 8 + (lane & 7);
    const int py = (int)(region / (unsigned)ra.tiles_x) * 4 + (lane >> 3);
    unsigned cnt = 0, nsteps = 0, last_row = 0;
    uint2* steps = ra.steps + (size_t)region * tp.view_steps;
    float T = 1.f;
    const bool ok = cgm::march_region(
        vd, cam, tp, px, py, T,
        [&](bool emit, unsigned ballot, float v0, float v1, float v2, float w, float G) {
            const unsigned n = __popc(ballot);
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(S.w + W_TAIL, n);
            base = __shfl_sync(0xffffffffu, base, 0);
            const unsigned t_last = (base + n - 1u) / 128u;
            // the ring slots of rows [base, base + n) must have been read
            bool free_ok = true;
            if (lane == 0)
                free_ok = spin_until(
                    S, [&] { return ld_volatile(S.w + W_RELEASED) + RT_RING > t_last; }, status);
            if (!__shfl_sync(0xffffffffu, free_ok, 0)) return false;
            if (emit) {
                const unsigned rank = __popc(ballot & ((1u << lane) - 1u));
                const unsigned row = base + rank;
                const unsigned at = row % (RT_RING * 128u);
                S.pos[at] = make_float4(v0, v1, v2, w);
                S.meta[at] = make_uint2(__float_as_uint(G), (ri << 16) | (cnt + rank));
                mbar_arrive(S.full + (row / 128u) % RT_RING, 1u);
            }
            if (lane == 0) steps[nsteps] = make_uint2(cnt, ballot);
            nsteps++;
            cnt += n;
            last_row = base + n - 1u;
            return true;
        });
    if (!ok) return false;
    rc.T[lane] = T;
    __syncwarp();
    if (lane == 0) {
        rc.nsteps = nsteps;
        rc.last_row = last_row;
        // the count last: the epilogue may already be counting this region
        st_volatile(&rc.count, cnt);
    }
    __syncwarp();
    return true;
}

template <int FMT>
__device__ __noinline__ float exact_tau(const VolDesc& vd, const ConeSchedule& cone, float x,
                                        float y, float z, const float* sun) {
    return cgs::sun_cone<FMT>(vd, cone, x, y, z, sun[0], sun[1], sun[2]);
}

template <int FMT>
__global__ void __launch_bounds__(RT_THREADS, RT_CTAS_PER_SM)
    k_render_mlp_tc(const __grid_constant__ VolDesc vd, const __grid_constant__ CamDesc cam,
                    const __grid_constant__ TraceParams tp, const __grid_constant__ ConeSchedule cone,
                    const __grid_constant__ MlpDev m, const __grid_constant__ FeatGeom geo,
                    RenderArgs ra, unsigned long long* status) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_addr(smem_raw);
    uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    Shared S;
    S.act = base + OFF_ACT;
    S.net = base + OFF_NET;
    S.pos = reinterpret_cast<float4*>(base + OFF_POS);
    S.meta = reinterpret_cast<uint2*>(base + OFF_META);
    S.rec = reinterpret_cast<Rec*>(base + OFF_REC);
    S.full = reinterpret_cast<uint64_t*>(base + OFF_BAR);
    S.act_ready = S.full + RT_RING;
    S.mma_done = S.full + RT_RING + 1;
    S.w = reinterpret_cast<unsigned*>(base + OFF_WORDS);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    mlptc::stage_network<MLP_MAX_LAYERS>(S.net, m, tid, RT_THREADS);
    for (int i = tid; i < RT_PRODUCERS * RT_RECS; i += RT_THREADS) S.rec[i].busy = 0u;
    // the shared words (not W_TMEM: the allocation below writes it)
    if (tid < W_COUNT && tid != W_TMEM) S.w[tid] = tid == W_END ? 0xFFFFFFFFu : 0u;
    if (tid == 0) {
        for (int i = 0; i < RT_RING; ++i) tc::mbar_init(S.full + i, 128);
        tc::mbar_init(S.act_ready, RT_EPI_WARPS);
        tc::mbar_init(S.mma_done, 1);
        tc::fence_mbar_init();
    }
    if (warp == RT_MMA_WARP) {
        tc::tmem_alloc(S.w + W_TMEM, RT_TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.w[W_TMEM];
    const float amb = tp.ambient;

    if (warp < RT_EPI_WARPS) {
        // ---- epilogue: one row of every tile per thread.  Every decision to
        // leave the loop is taken jointly by the four warps (bar.red) at the
        // top of a tile, so they always meet at the same barriers.
        const uint32_t dw = tmem + ((uint32_t)(warp * 32) << 16);
        unsigned n_fallback = 0, n_valid = 0, mphase = 0;
        bool bad = false;  // a wait of this warp ran out or the CTA aborts
        for (unsigned t = 0;; ++t) {
            const unsigned slot = t % RT_RING;
            bool stop = bad || !wait_phase(S, S.full + slot, (t / RT_RING) & 1u, status) ||
                        t == ld_volatile(S.w + W_END);
            if (epi_any(stop)) break;
            // every row of the tile is read: release the slot to the producers
            const float4 sp = S.pos[slot * 128 + tid];
            const uint2 mt = S.meta[slot * 128 + tid];
            epi_sync();
            if (tid == 0) st_volatile(S.w + W_RELEASED, t + 1u);
            const unsigned ri = mt.y >> 16;
            const bool valid = ri != RT_NO_REC;
            float f[MLP_IN];
            float tau_fb = -1.f;
            if (valid) {
                mlp::features(geo, sp.x, sp.y, sp.z, tp.sun[0], tp.sun[1], tp.sun[2], f);
                if (!mlp::in_range(m, f)) tau_fb = exact_tau<FMT>(vd, cone, sp.x, sp.y, sp.z, tp.sun);
            }
            mlptc::write_inputs(S.act, tid, m, f, valid);
            float y = 0.f;
#pragma unroll 1
            for (int layer = 0; layer < m.layers && !bad; ++layer) {
                // this warp's activation rows -> visible to the tensor core
                tc::fence_proxy_async();
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(S.act_ready, 1u);
                bad = !__all_sync(0xffffffffu, wait_phase(S, S.mma_done, mphase, status));
                if (bad) break;
                mphase ^= 1u;
                tc::fence_after_sync();
                const bool last = layer == m.layers - 1;
                const float yy = mlptc::layer_epilogue(last, dw, S.act, tid, m);
                if (last) y = yy;
            }
            if (bad) continue;  // leaves at the next tile's joint decision
            if (valid) {
                n_valid++;
                float tau;
                if (tau_fb >= 0.f) {
                    tau = tau_fb;
                    n_fallback++;
                } else {
                    tau = m.tau_scale * mlp::softplus(y);
                }
                const Rec& rc = S.rec[ri];
                const size_t at = (size_t)rc.region * ra.cap + (mt.y & 0xFFFFu);
                if (CG_IN_BOUNDS(at, (size_t)ra.regions * ra.cap))
                    ra.contrib[at] = sp.w * __expf(-tp.sigma * tau) *
                                     (amb + (1.f - amb) * __uint_as_float(mt.x));
            }
            // count the shaded samples per record (rows of one record share
            // one atomic)
            __threadfence_block();
            const unsigned key = valid ? ri : 0xFFFFFFFFu;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            if (valid && lane == __ffs(peers) - 1) atomicAdd(&S.rec[ri].done, (unsigned)__popc(peers));
        }
        // stop the issuer: the flag, then one more arrival per warp
        if (tid == 0) st_volatile(S.w + W_STOP, 1u);
        __syncwarp();
        if (lane == 0) mbar_arrive(S.act_ready, 1u);
        unsigned tot = n_fallback, nv = n_valid;
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
            nv += __shfl_xor_sync(0xffffffffu, nv, o);
        }
        if (lane == 0) {
            if (tot) atomicAdd(status, (unsigned long long)tot);
            if (nv) atomicAdd(status + 2, (unsigned long long)nv);
        }
    } else if (warp == RT_MMA_WARP) {
        // ---- tensor-core issue: m.layers layers per tile until told to stop
        const uint32_t a_addr = tc::smem_addr(S.act), net_addr = tc::smem_addr(S.net);
        unsigned aphase = 0, issued = 0;
        for (;;) {
            bool ok = true;
            if (lane == 0) ok = wait_phase(S, S.act_ready, aphase, status);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            aphase ^= 1u;
            if (ld_volatile(S.w + W_STOP) || ld_volatile(S.w + W_ABORT)) break;
            tc::fence_after_sync();
            if (lane == 0)
                mlptc::issue_layer<MLP_MAX_LAYERS>((int)(issued % (unsigned)m.layers), tmem, a_addr,
                                                   net_addr,
                                   S.mma_done);
            issued++;
            __syncwarp();
        }
        // an abort may leave the last commit unobserved: drain it (bounded)
        if (issued && ld_volatile(S.w + W_ABORT)) {
            bool drained = true;
            if (lane == 0) drained = tc::mbar_wait(S.mma_done, (issued - 1u) & 1u, RT_WAIT_NS);
            drained = __shfl_sync(0xffffffffu, drained, 0);
            if (!drained && lane == 0) atomicOr(status + 1, 3ull);
        }
    } else {
        // ---- producers: march regions, composite them once shaded
        const int p = warp - RT_FIRST_PRODUCER;
        Rec* recs = S.rec + p * RT_RECS;
        unsigned r = 0;
        bool ok = true;
        for (;;) {
            Rec& rc = recs[r];
            if (rc.busy) {
                ok = finish_region(S, rc, ra, cam, tp, tp.view_steps, status);
                if (!ok) break;
            }
            unsigned region = 0;
            if (lane == 0) region = (unsigned)atomicAdd(status + 3, 1ull);
            region = __shfl_sync(0xffffffffu, region, 0);
            if (region >= (unsigned)ra.regions) break;
            if (lane == 0) {
                rc.region = region;
                rc.done = 0u;
                rc.count = RT_IN_PROGRESS;
                rc.busy = 1u;
                __threadfence_block();  // before any of the region's rows is published
            }
            __syncwarp();
            ok = march_region(S, rc, (unsigned)(p * RT_RECS) + r, region, vd, cam, tp, ra, status);
            if (!ok) break;
            r = (r + 1u) % RT_RECS;
        }
        // the remaining regions, oldest first
        for (int k = 0; k < RT_RECS && ok; ++k) {
            Rec& rc = recs[(r + k) % RT_RECS];
            if (rc.busy) ok = finish_region(S, rc, ra, cam, tp, tp.view_steps, status);
        }
        // the last producer marks the end: the tile after the last one
        unsigned last = 0;
        if (lane == 0) last = atomicAdd(S.w + W_PDONE, 1u) == RT_PRODUCERS - 1;
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last && lane == 0) {
            const unsigned tail = ld_volatile(S.w + W_TAIL);
            const unsigned e = (tail + 127u) / 128u;
            if (!ld_volatile(S.w + W_ABORT) &&
                spin_until(S, [&] { return ld_volatile(S.w + W_RELEASED) + RT_RING > e; }, status)) {
                st_volatile(S.w + W_END, e);
                mbar_arrive(S.full + e % RT_RING, 128u);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == RT_MMA_WARP) tc::tmem_dealloc(tmem, RT_TMEM_COLS);
}

}  // namespace

cudaError_t launch_render_mlp_tc(VolDesc vd, CamDesc cam, TraceParams tp, const MlpDev& m,
                                 float* contrib, uint2* steps, float4* dst,
                                 unsigned long long* status, cudaStream_t st) {
    if (m.layers < 1 || m.layers > MLP_MAX_LAYERS) return cudaErrorInvalidValue;
    const ConeSchedule cone = make_cone_schedule(vd, tp);
    const FeatGeom geo = feat_geom(vd, m);
    RenderArgs ra;
    ra.contrib = contrib;
    ra.steps = steps;
    ra.dst = dst;
    ra.tiles_x = (cam.W + 7) / 8;
    ra.regions = ra.tiles_x * ((cam.H + 3) / 4);
    ra.cap = 32 * tp.view_steps;
    // the shared-memory attribute and the grid are set once per device
    static std::atomic<int> grid[2][64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const int f = vd.fmt == 0 ? 0 : 1;
    if (!grid[f][dev].load(std::memory_order_acquire)) {
        const void* fn = f == 0 ? (const void*)k_render_mlp_tc<0> : (const void*)k_render_mlp_tc<1>;
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, RT_SMEM_BYTES);
        if (e != cudaSuccess) return e;
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        grid[f][dev].store(sms * RT_CTAS_PER_SM, std::memory_order_release);
    }
    const int blocks = grid[f][dev].load(std::memory_order_acquire);
    if (f == 0)
        k_render_mlp_tc<0><<<blocks, RT_THREADS, RT_SMEM_BYTES, st>>>(vd, cam, tp, cone, m, geo, ra,
                                                                       status);
    else
        k_render_mlp_tc<1><<<blocks, RT_THREADS, RT_SMEM_BYTES, st>>>(vd, cam, tp, cone, m, geo, ra,
                                                                       status);
    return cudaGetLastError();
}

CG_OOB_TU(k_render_tc)
