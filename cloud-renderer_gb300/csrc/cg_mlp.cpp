// cg_mlp.cpp -- the MLP sun-transmittance surrogate behind the C ABI:
// creation, configuration, features, inference, gradient evaluation,
// training (CUDA-graph replay of the fused step + Adam) and checkpoints.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cg_host_util.h"

struct cg_mlp {
    cg_context* ctx = nullptr;
    DevBuf params, w16, m, v, step, ticket, partial, loss, grad;
    DevBuf status;  // the training kernels' status word (see TrainArgs)
    int layers = MLP_DEFAULT_LAYERS;  // hidden layers, fixed at creation
    cg_mlp_config cfg{};
    int host_step = 0;
    MlpConsts consts{};  // host copy of the biases / output row (see MlpConsts)
};

namespace {

// SplitMix64 (Steele, Lea & Flood 2014) for the weight initialisation.
struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Crc32Table {
    uint32_t t[256];
    Crc32Table() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const void* data, size_t n) {
    static const Crc32Table tab;  // initialised once, thread-safe
    const uint32_t* table = tab.t;
    const uint8_t* p = reinterpret_cast<const uint8_t*>(data);
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

// FP16 weight image of a parameter vector (W4 rows 1-7 zero).
void half_image(const float* p, std::vector<__half>& h) {
    h.assign(MLP_NHALF, __float2half(0.f));
    for (int i = 0; i < 1024; ++i) h[MLP_H_W1 + i] = __float2half(p[MLP_W1 + i]);
    for (int i = 0; i < 4096; ++i) h[MLP_H_W2 + i] = __float2half(p[MLP_W2 + i]);
    for (int i = 0; i < 4096; ++i) h[MLP_H_W3 + i] = __float2half(p[MLP_W3 + i]);
    for (int i = 0; i < 64; ++i) h[MLP_H_W4 + i] = __float2half(p[MLP_W4 + i]);
}

void set_consts(cg_mlp* m, const float* b1, const float* b2, const float* b3, const float* w4,
                float b4) {
    for (int i = 0; i < MLP_H; ++i) {
        m->consts.hb[i] = 0.5f * b1[i];
        m->consts.hb[MLP_H + i] = 0.5f * b2[i];
        m->consts.hb[2 * MLP_H + i] = 0.5f * b3[i];
        m->consts.w4[i] = __half2float(__float2half(w4[i]));
    }
    m->consts.b4 = b4;
}

// Zero the blocks of the hidden layers a model of `layers` does not use.
void zero_frozen(int layers, float* p) {
    int lo, hi;
    mlp_frozen_range(layers, lo, hi);
    for (int i = lo; i < hi; ++i) p[i] = 0.f;
}

cg_status upload_params(cg_mlp* m, const float* src) {
    std::vector<float> p(src, src + MLP_NPARAM);
    zero_frozen(m->layers, p.data());
    std::vector<__half> h;
    half_image(p.data(), h);
    set_consts(m, &p[MLP_B1], &p[MLP_B2], &p[MLP_B3], &p[MLP_W4], p[MLP_B4]);
    CG_CUDA(cudaMemcpy(m->params.p, p.data(), MLP_NPARAM * 4, cudaMemcpyHostToDevice));
    CG_CUDA(cudaMemcpy(m->w16.p, h.data(), MLP_NHALF * 2, cudaMemcpyHostToDevice));
    return CG_OK;
}

MlpDev device_view(const cg_mlp* m) {
    MlpDev d;
    d.params = m->params.as<const float>();
    d.w16 = m->w16.as<const __half>();
    for (int j = 0; j < MLP_IN; ++j) {
        d.mu[j] = m->cfg.mean[j];
        d.inv_sd[j] = m->cfg.stddev[j] > 0.f ? 1.f / m->cfg.stddev[j] : 1.f;
        d.fmin[j] = m->cfg.feature_min[j];
        d.fmax[j] = m->cfg.feature_max[j];
    }
    d.tau_scale = m->cfg.tau_scale;
    d.h0 = m->cfg.initial_height;
    d.lb = m->cfg.base_level;
    d.layers = m->layers;
    d.k = m->consts;
    return d;
}

bool cfg_ok(const cg_mlp_config* c) {
    if (c->base_level < 0 || c->base_level > 12) return false;
    if (!std::isfinite(c->initial_height) || !std::isfinite(c->tau_scale) || !(c->tau_scale > 0.f))
        return false;
    for (int j = 0; j < MLP_IN; ++j)
        if (!std::isfinite(c->mean[j]) || !std::isfinite(c->stddev[j]) || !(c->stddev[j] > 0.f) ||
            std::isnan(c->feature_min[j]) || std::isnan(c->feature_max[j]))
            return false;
    return true;
}

}  // namespace

extern "C" void cg_mlp_config_default(cg_mlp_config* c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->base_level = 2;
    c->initial_height = 1.0f;
    c->dimension = 256;
    c->sun_steps = 24;
    c->cone_half_angle = 0.03f;
    c->cone_initial_height = 1.0f;
    c->cone_min_radius = 2.0f;
    c->lod_offset = 0.0f;
    for (int j = 0; j < MLP_IN; ++j) {
        c->mean[j] = 0.f;
        c->stddev[j] = 1.f;
        c->feature_min[j] = -INFINITY;
        c->feature_max[j] = INFINITY;
    }
    c->tau_scale = 1.0f;
}

extern "C" int cg_mlp_param_count(void) { return MLP_NPARAM; }

extern "C" cg_status cg_mlp_create(cg_context* ctx, uint64_t seed, cg_mlp** out) {
    return cg_mlp_create_layers(ctx, seed, MLP_DEFAULT_LAYERS, out);
}

extern "C" int cg_mlp_hidden_layers(const cg_mlp* m) { return m ? m->layers : 0; }

extern "C" cg_status cg_mlp_create_layers(cg_context* ctx, uint64_t seed, int hidden_layers,
                                          cg_mlp** out) {
    CG_CHECK(ctx && out, CG_ERR_INVALID_ARGUMENT, "cg_mlp_create: null pointer");
    *out = nullptr;
    CG_CHECK(hidden_layers >= 1 && hidden_layers <= MLP_MAX_LAYERS, CG_ERR_OUT_OF_RANGE,
             "cg_mlp_create: hidden_layers %d not in [1, %d]", hidden_layers, MLP_MAX_LAYERS);
    CG_CUDA(cudaSetDevice(ctx->device));
    cg_mlp* m = new cg_mlp();
    m->ctx = ctx;
    m->layers = hidden_layers;
    context_retain(ctx);
    cg_mlp_config_default(&m->cfg);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = m->params.ensure(MLP_NPARAM * 4);
    if (e == cudaSuccess) e = m->w16.ensure(MLP_NHALF * 2);
    if (e == cudaSuccess) e = m->m.ensure(MLP_NPARAM * 4);
    if (e == cudaSuccess) e = m->v.ensure(MLP_NPARAM * 4);
    if (e == cudaSuccess) e = m->step.ensure(16);
    if (e == cudaSuccess) e = m->ticket.ensure(16);
    if (e == cudaSuccess) e = m->grad.ensure((MLP_NPARAM + 1) * 4);
    if (e == cudaSuccess) e = m->status.ensure(16);
    if (e == cudaSuccess) e = cudaMemset(m->status.p, 0, 16);
    if (e == cudaSuccess) e = cudaMemset(m->m.p, 0, MLP_NPARAM * 4);
    if (e == cudaSuccess) e = cudaMemset(m->v.p, 0, MLP_NPARAM * 4);
    if (e == cudaSuccess) e = cudaMemset(m->step.p, 0, 16);
    if (e == cudaSuccess) e = cudaMemset(m->ticket.p, 0, 16);
    if (e != cudaSuccess) {
        cg_mlp_destroy(m);
        return fail(CG_ERR_OUT_OF_MEMORY, "cg_mlp_create: %s", cudaGetErrorString(e));
    }
    // uniform(-b, b) with b = sqrt(6 / fan_in) (He-uniform); output layer
    // b = sqrt(3 / fan_in); biases zero
    std::vector<float> p(MLP_NPARAM, 0.f);
    SplitMix64 r{seed};
    auto fill = [&](int off, int n, int fan_in, double gain) {
        const double b = std::sqrt(gain / fan_in);
        for (int i = 0; i < n; ++i) p[off + i] = (float)((2.0 * r.uniform() - 1.0) * b);
    };
    // (the stream draws all three hidden layers, so a layer's initial weights
    // do not depend on the depth; the unused ones are zeroed on upload)
    fill(MLP_W1, 1024, 16, 6.0);
    fill(MLP_W2, 4096, 64, 6.0);
    fill(MLP_W3, 4096, 64, 6.0);
    fill(MLP_W4, 64, 64, 3.0);
    cg_status st = upload_params(m, p.data());
    if (st != CG_OK) {
        cg_mlp_destroy(m);
        return st;
    }
    *out = m;
    return CG_OK;
}

extern "C" void cg_mlp_destroy(cg_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->ctx->device);
    cudaStreamSynchronize(m->ctx->stream);
    DevBuf* bufs[] = {&m->params, &m->w16, &m->m, &m->v, &m->step, &m->ticket,
                      &m->partial, &m->loss, &m->grad, &m->status};
    for (DevBuf* b : bufs) b->release();
    cg_context* ctx = m->ctx;
    delete m;
    context_release(ctx);
}

extern "C" cg_status cg_mlp_configure(cg_mlp* m, const cg_mlp_config* c) {
    CG_CHECK(m && c, CG_ERR_INVALID_ARGUMENT, "cg_mlp_configure: null pointer");
    CG_CHECK(cfg_ok(c), CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_configure: base_level in [0,12], finite values, stddev and tau_scale > 0");
    m->cfg = *c;
    return CG_OK;
}

extern "C" cg_status cg_mlp_get_config(const cg_mlp* m, cg_mlp_config* c) {
    CG_CHECK(m && c, CG_ERR_INVALID_ARGUMENT, "cg_mlp_get_config: null pointer");
    *c = m->cfg;
    return CG_OK;
}

// Surrogate view for a render; the model must have been trained for this
// volume resolution and sun-cone configuration.
cg_status mlp_device_for_render(const cg_mlp* m, const cg_volume* v, const cg_render_params* p,
                                MlpDev& md) {
    CG_CHECK(m, CG_ERR_INVALID_ARGUMENT, "render params: use_mlp set without an mlp");
    CG_CHECK(m->ctx == v->ctx, CG_ERR_INVALID_ARGUMENT, "render params: mlp of another context");
    const cg_mlp_config& c = m->cfg;
    CG_CHECK(c.dimension == v->D && c.sun_steps == p->sun_steps &&
                 c.cone_half_angle == p->cone_half_angle &&
                 c.cone_initial_height == p->cone_initial_height &&
                 c.cone_min_radius == p->cone_min_radius && c.lod_offset == p->lod_offset &&
                 p->cone_mode == CG_CONE_TRANSMITTANCE,
             CG_ERR_INVALID_ARGUMENT,
             "render params: the surrogate was trained for dimension %d and a %d-step "
             "transmittance cone (half-angle %g, h0 %g, rmin %g, lod offset %g)",
             c.dimension, c.sun_steps, (double)c.cone_half_angle, (double)c.cone_initial_height,
             (double)c.cone_min_radius, (double)c.lod_offset);
    md = device_view(m);
    return CG_OK;
}

cg_status ensure_samples(cg_context* ctx, int width, int height, int view_steps, SampleBuf& sb) {
    const size_t tiles = (size_t)((width + 15) / 16) * ((height + 15) / 16);
    const size_t regions = tiles * 8;
    const size_t cap = (size_t)32 * view_steps;
    const size_t n = regions * cap;
    CG_CHECK(n < (size_t)0xFFFFFFFFu, CG_ERR_OUT_OF_RANGE,
             "render: %zu sample slots (pixels x view_steps) exceed 2^32", n);
    // counts, step counts, flat total, step tables (2 words each), flat slots
    // (the padded flat order has at most 31 padding rows per 8 regions)
    const size_t flat = n + 32 * (regions / 8 + 1);
    const size_t idx_words = 2 * regions + 2 + 2 * regions * view_steps + 2 + flat;
    const size_t pixels = (size_t)width * height;
    if (ctx->samples_pw.bytes < n * 16 || ctx->samples_gl.bytes < n * 8 ||
        ctx->samples_c.bytes < n * 4 || ctx->samples_cnt.bytes < idx_words * 4 ||
        ctx->samples_alpha.bytes < pixels * 4) {
        CG_CUDA(cudaStreamSynchronize(ctx->stream));
        CG_CUDA(ctx->samples_pw.ensure(n * 16));
        CG_CUDA(ctx->samples_gl.ensure(n * 8));
        CG_CUDA(ctx->samples_c.ensure(n * 4));
        CG_CUDA(ctx->samples_cnt.ensure(idx_words * 4));
        CG_CUDA(ctx->samples_alpha.ensure(pixels * 4));
    }
    CG_CUDA(ctx->fallbacks.ensure(32));
    sb.pos_w = ctx->samples_pw.as<float4>();
    sb.light_lane = ctx->samples_gl.as<float2>();
    sb.contrib = ctx->samples_c.as<float>();
    sb.alpha = ctx->samples_alpha.as<float>();
    sb.count = ctx->samples_cnt.as<unsigned>();
    sb.nsteps = sb.count + regions;
    sb.flat_total = sb.nsteps + regions;
    // 8-byte aligned start for the (slot, ballot) pairs
    size_t at = (size_t)(sb.flat_total + 1 - ctx->samples_cnt.as<unsigned>());
    at = (at + 1) & ~(size_t)1;
    sb.steps = reinterpret_cast<uint2*>(ctx->samples_cnt.as<unsigned>() + at);
    sb.slot_of = ctx->samples_cnt.as<unsigned>() + at + 2 * regions * (size_t)view_steps;
    sb.capacity = (int)cap;
    sb.nslots = n;
    return CG_OK;
}

cg_status ensure_render_slots(cg_context* ctx, int width, int height, int view_steps,
                              float*& contrib, uint2*& steps) {
    const size_t regions = (size_t)((width + 7) / 8) * ((height + 3) / 4);
    const size_t n = regions * (size_t)32 * view_steps;
    CG_CHECK(n < (size_t)0xFFFFFFFFu, CG_ERR_OUT_OF_RANGE,
             "render: %zu sample slots (pixels x view_steps) exceed 2^32", n);
    const size_t step_words = 2 * regions * (size_t)view_steps;
    if (ctx->samples_c.bytes < n * 4 || ctx->samples_cnt.bytes < step_words * 4) {
        CG_CUDA(cudaStreamSynchronize(ctx->stream));
        CG_CUDA(ctx->samples_c.ensure(n * 4));
        CG_CUDA(ctx->samples_cnt.ensure(step_words * 4));
    }
    CG_CUDA(ctx->fallbacks.ensure(32));
    contrib = ctx->samples_c.as<float>();
    steps = reinterpret_cast<uint2*>(ctx->samples_cnt.as<unsigned>());
    return CG_OK;
}

extern "C" cg_status cg_context_mlp_fallbacks(cg_context* ctx, uint64_t* out) {
    CG_CHECK(ctx && out, CG_ERR_INVALID_ARGUMENT, "cg_context_mlp_fallbacks: null pointer");
    *out = 0;
    if (!ctx->fallbacks.p) return CG_OK;
    CG_CUDA(cudaSetDevice(ctx->device));
    CG_CUDA(cudaDeviceSynchronize());
    unsigned long long h[2] = {0, 0};
    CG_CUDA(cudaMemcpy(h, ctx->fallbacks.p, 16, cudaMemcpyDeviceToHost));
    *out = h[0];
    CG_CHECK((h[1] & 2ull) == 0, CG_ERR_DEVICE_FAULT,
             "surrogate render: a tensor-core wait ran out of its time limit (1 s) and the "
             "drain after it did not complete; the device must be treated as faulted");
    CG_CHECK(h[1] == 0, CG_ERR_DEVICE_FAULT,
             "surrogate render: a tensor-core wait ran out of its time limit (1 s)");
    return CG_OK;
}

extern "C" cg_status cg_context_check_wait_timeout(cg_context* ctx, uint32_t limit_us,
                                                   uint64_t* waited_us) {
    CG_CHECK(ctx && waited_us, CG_ERR_INVALID_ARGUMENT,
             "cg_context_check_wait_timeout: null pointer");
    CG_CHECK(limit_us >= 1 && limit_us <= 1000000, CG_ERR_OUT_OF_RANGE,
             "cg_context_check_wait_timeout: limit %u us not in [1, 1e6]", limit_us);
    CG_CUDA(cudaSetDevice(ctx->device));
    CG_CUDA(ctx->fallbacks.ensure(32));
    cudaStream_t s = ctx->stream;
    CG_CUDA(cudaMemsetAsync(ctx->fallbacks.p, 0, 32, s));
    CG_LAUNCH(ctx, launch_wait_probe((uint64_t)limit_us * 1000ull,
                                     ctx->fallbacks.as<unsigned long long>(), s));
    CG_CUDA(cudaStreamSynchronize(s));
    unsigned long long h[4] = {0, 0, 0, 0};
    CG_CUDA(cudaMemcpy(h, ctx->fallbacks.p, 32, cudaMemcpyDeviceToHost));
    *waited_us = h[3] / 1000ull;
    ctx->shaded_valid = false;
    CG_CHECK(h[1] == 0, CG_ERR_DEVICE_FAULT,
             "wait probe: the bounded mbarrier wait ran out after %llu us, as it must",
             (unsigned long long)(h[3] / 1000ull));
    return CG_OK;
}

// Stage host inputs on the device when needed (tmp receives the copy).
static cg_status stage_in(const float* src, size_t n, int on_device, DevBuf& tmp, const float*& dst,
                          cudaStream_t s) {
    if (on_device) {
        dst = src;
        return CG_OK;
    }
    CG_CUDA(tmp.ensure(n * 4));
    CG_CUDA(cudaMemcpyAsync(tmp.p, src, n * 4, cudaMemcpyHostToDevice, s));
    dst = tmp.as<const float>();
    return CG_OK;
}

extern "C" cg_status cg_mlp_features(const cg_volume* v, const cg_mlp* m, const float* positions,
                                     int n, const float direction[3], float* out, int on_device,
                                     void* stream) {
    CG_CHECK(v && m && direction && (n == 0 || (positions && out)), CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_features: null pointer");
    CG_CHECK(n >= 0, CG_ERR_OUT_OF_RANGE, "cg_mlp_features: n < 0");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_mlp_features: volume has not been voxelized");
    if (n == 0) return CG_OK;
    double dn = std::sqrt((double)direction[0] * direction[0] +
                          (double)direction[1] * direction[1] +
                          (double)direction[2] * direction[2]);
    CG_CHECK(std::isfinite(dn) && dn > 0.0, CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_features: direction must be finite and non-zero");
    float dir[3] = {(float)(direction[0] / dn), (float)(direction[1] / dn),
                    (float)(direction[2] / dn)};
    cg_context* ctx = v->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    DevBuf tin, tout;
    const float* dpos;
    cg_status st = stage_in(positions, (size_t)n * 3, on_device, tin, dpos, s);
    if (st != CG_OK) return st;
    float* dout = out;
    if (!on_device) {
        CG_CUDA(tout.ensure((size_t)n * MLP_IN * 4));
        dout = tout.as<float>();
    }
    st = ensure_textures(const_cast<cg_volume*>(v), s);
    if (st != CG_OK) return st;
    CG_LAUNCH(ctx, launch_mlp_features(desc_of(v), device_view(m), dpos, n, dir, dout, s));
    if (!on_device) {
        CG_CUDA(cudaMemcpyAsync(out, dout, (size_t)n * MLP_IN * 4, cudaMemcpyDeviceToHost, s));
        CG_CUDA(cudaStreamSynchronize(s));
    }
    return CG_OK;
}

extern "C" cg_status cg_mlp_infer(const cg_mlp* m, const float* features, int n, float* out,
                                  int on_device, void* stream) {
    CG_CHECK(m && (n == 0 || (features && out)), CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_infer: null pointer");
    CG_CHECK(n >= 0, CG_ERR_OUT_OF_RANGE, "cg_mlp_infer: n < 0");
    if (n == 0) return CG_OK;
    cg_context* ctx = m->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    DevBuf tin, tout;
    const float* df;
    cg_status st = stage_in(features, (size_t)n * MLP_IN, on_device, tin, df, s);
    if (st != CG_OK) return st;
    float* dout = out;
    if (!on_device) {
        CG_CUDA(tout.ensure((size_t)n * 4));
        dout = tout.as<float>();
    }
    // the tensor-core status block: [1] records a wait that ran out
    CG_CUDA(ctx->fallbacks.ensure(32));
    CG_CUDA(cudaMemsetAsync(ctx->fallbacks.p, 0, 32, s));
    ctx->shaded_valid = false;
    CG_LAUNCH(ctx, launch_mlp_infer(device_view(m), df, n, dout,
                                    ctx->fallbacks.as<unsigned long long>(), s));
    if (!on_device) {
        CG_CUDA(cudaMemcpyAsync(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
        unsigned long long h[2] = {0, 0};
        CG_CUDA(cudaMemcpyAsync(h, ctx->fallbacks.p, 16, cudaMemcpyDeviceToHost, s));
        CG_CUDA(cudaStreamSynchronize(s));
        CG_CHECK(h[1] == 0, CG_ERR_DEVICE_FAULT,
                 "cg_mlp_infer: a tensor-core wait ran out of its time limit (1 s)");
    }
    return CG_OK;
}

// the bound of every training-kernel wait (a wait longer than this is a fault)
static const unsigned long long kTrainWaitNs = 1000000000ull;

static TrainArgs train_args(const cg_mlp* m, const float* feat, const float* tau, long long n,
                            float sigma) {
    TrainArgs ta{};
    ta.feat = feat;
    ta.tau = tau;
    ta.N = n;
    MlpDev d = device_view(m);
    for (int j = 0; j < MLP_IN; ++j) {
        ta.mu[j] = d.mu[j];
        ta.inv_sd[j] = d.inv_sd[j];
    }
    ta.tau_scale = m->cfg.tau_scale;
    ta.sigma = sigma;
    ta.params = m->params.as<const float>();
    ta.w16 = m->w16.as<const __half>();
    ta.partial = m->partial.as<float>();
    ta.status = m->status.as<unsigned long long>();
    ta.wait_ns = kTrainWaitNs;
    ta.stall = 0;
    ta.layers = m->layers;
    return ta;
}

// The training kernels' status word after the stream has drained: CG_OK, or
// CG_ERR_DEVICE_FAULT naming what stopped (no update was made from the
// failing step on).
static cg_status train_status(cg_mlp* m, const char* who) {
    unsigned long long st = 0;
    CG_CUDA(cudaMemcpy(&st, m->status.p, 8, cudaMemcpyDeviceToHost));
    if (st == 0) return CG_OK;
    if (st & 4ull)
        return fail(CG_ERR_DEVICE_FAULT,
                    "%s: the fused optimiser's grid barrier ran out of its time limit; the "
                    "update of that step may be partial", who);
    if (st & 2ull)
        return fail(CG_ERR_DEVICE_FAULT,
                    "%s: a tensor-core wait ran out of its time limit and the drain after it "
                    "did not complete; no update was made from that step on and the device "
                    "must be treated as faulted", who);
    return fail(CG_ERR_DEVICE_FAULT,
                "%s: a tensor-core wait ran out of its time limit; no update was made from "
                "that step on", who);
}

extern "C" cg_status cg_mlp_gradient(cg_mlp* m, const float* features, const float* tau, int n,
                                     float sigma, float* grad, float* loss, int on_device) {
    CG_CHECK(m && features && tau && grad && loss, CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_gradient: null pointer");
    CG_CHECK(n >= 1 && n <= (1 << 22), CG_ERR_OUT_OF_RANGE, "cg_mlp_gradient: n not in [1, 2^22]");
    CG_CHECK(std::isfinite(sigma) && sigma > 0.f, CG_ERR_INVALID_ARGUMENT,
             "cg_mlp_gradient: sigma must be > 0");
    cg_context* ctx = m->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    DevBuf tf, tt;
    const float *df, *dt;
    cg_status st = stage_in(features, (size_t)n * MLP_IN, on_device, tf, df, s);
    if (st != CG_OK) return st;
    st = stage_in(tau, (size_t)n, on_device, tt, dt, s);
    if (st != CG_OK) return st;
    const int ctas = (n + 127) / 128;
    CG_CUDA(cudaStreamSynchronize(s));
    CG_CUDA(m->partial.ensure((size_t)ctas * (MLP_NPARAM + 1) * 4));
    CG_CUDA(cudaMemsetAsync(m->status.p, 0, 16, s));
    TrainArgs ta = train_args(m, df, dt, n, sigma);
    ta.sequential = 1;
    ta.offset = 0;
    ta.batch = ctas * 128;
    CG_LAUNCH(ctx, launch_mlp_train(ta, ctas, s));
    AdamArgs aa{};
    aa.partial = m->partial.as<const float>();
    aa.nparts = ctas;
    aa.inv_batch = 1.f / (float)n;
    aa.grad_out = m->grad.as<float>();
    aa.loss_out = m->grad.as<float>() + MLP_NPARAM;
    aa.status = m->status.as<const unsigned long long>();
    mlp_frozen_range(m->layers, aa.frozen_lo, aa.frozen_hi);
    CG_LAUNCH(ctx, launch_mlp_adam(aa, s));
    std::vector<float> h(MLP_NPARAM + 1);
    CG_CUDA(cudaMemcpyAsync(h.data(), m->grad.p, (MLP_NPARAM + 1) * 4, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    st = train_status(m, "cg_mlp_gradient");
    if (st != CG_OK) return st;
    memcpy(grad, h.data(), MLP_NPARAM * 4);
    *loss = h[MLP_NPARAM];
    return CG_OK;
}

static unsigned long long gcd_u64(unsigned long long a, unsigned long long b) {
    while (b) {
        unsigned long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

extern "C" void cg_train_params_default(cg_train_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->steps = 20000;
    p->batch = 16384;
    p->lr = 1e-3f;
    p->beta1 = 0.9f;
    p->beta2 = 0.999f;
    p->eps = 1e-8f;
    p->sigma = 2.0f;
    p->seed = 1;
}

// Training: `steps` fused steps (forward + backward, one CTA per 128 rows,
// then the ordered gradient reduction with Adam), replayed from a CUDA graph
// of up to 50 steps.  Batches walk a multiplicative permutation of the
// dataset.  loss_per_step (host, may be NULL) receives the mean loss of
// every step.
static cg_status train_impl(cg_mlp* m, const float* d_features, const float* d_tau, long long n,
                            const cg_train_params* tp, float* loss_per_step,
                            unsigned long long wait_ns, int stall);

extern "C" cg_status cg_mlp_train(cg_mlp* m, const float* d_features, const float* d_tau,
                                  long long n, const cg_train_params* tp, float* loss_per_step) {
    return train_impl(m, d_features, d_tau, n, tp, loss_per_step, kTrainWaitNs, 0);
}

extern "C" cg_status cg_mlp_check_train_timeout(cg_mlp* m, const float* d_features,
                                                const float* d_tau, long long n, int steps,
                                                uint32_t limit_us) {
    CG_CHECK(m, CG_ERR_INVALID_ARGUMENT, "cg_mlp_check_train_timeout: null pointer");
    CG_CHECK(limit_us >= 1 && limit_us <= 1000000, CG_ERR_OUT_OF_RANGE,
             "cg_mlp_check_train_timeout: limit %u us not in [1, 1e6]", limit_us);
    CG_CHECK(steps >= 1 && steps <= 50, CG_ERR_OUT_OF_RANGE,
             "cg_mlp_check_train_timeout: steps not in [1, 50]");
    cg_train_params tp;
    cg_train_params_default(&tp);
    tp.steps = steps;
    tp.batch = 1024;
    return train_impl(m, d_features, d_tau, n, &tp, nullptr, (unsigned long long)limit_us * 1000ull,
                      1);
}

static cg_status train_impl(cg_mlp* m, const float* d_features, const float* d_tau, long long n,
                            const cg_train_params* tp, float* loss_per_step,
                            unsigned long long wait_ns, int stall) {
    NvtxRange nvtx_("cg_mlp_train");
    CG_CHECK(m && d_features && d_tau && tp, CG_ERR_INVALID_ARGUMENT, "cg_mlp_train: null pointer");
    CG_CHECK(n >= 1 && n <= (1ll << 31), CG_ERR_OUT_OF_RANGE, "cg_mlp_train: n not in [1, 2^31]");
    CG_CHECK(tp->steps >= 0 && tp->steps <= 10000000, CG_ERR_OUT_OF_RANGE,
             "cg_mlp_train: steps not in [0, 1e7]");
    CG_CHECK(tp->batch >= 128 && tp->batch <= (1 << 20) && tp->batch % 128 == 0,
             CG_ERR_OUT_OF_RANGE, "cg_mlp_train: batch must be a multiple of 128 in [128, 2^20]");
    CG_CHECK(std::isfinite(tp->lr) && tp->lr > 0.f && tp->beta1 >= 0.f && tp->beta1 < 1.f &&
                 tp->beta2 >= 0.f && tp->beta2 < 1.f && tp->eps > 0.f && tp->sigma > 0.f,
             CG_ERR_INVALID_ARGUMENT, "cg_mlp_train: bad optimiser parameters");
    if (tp->steps == 0) return CG_OK;
    cg_context* ctx = m->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int ctas = tp->batch / 128;
    CG_CUDA(cudaStreamSynchronize(s));
    CG_CUDA(m->partial.ensure((size_t)ctas * (MLP_NPARAM + 1) * 4));
    CG_CUDA(m->loss.ensure((size_t)tp->steps * 4));
    // multiplier coprime with n, from the seed
    static const unsigned long long primes[] = {2654435761ull, 2246822519ull, 3266489917ull,
                                                668265263ull, 374761393ull, 1610612741ull};
    unsigned long long mul = primes[tp->seed % 6];
    while (gcd_u64(mul, (unsigned long long)n) != 1ull) mul += 2;
    CG_CUDA(cudaMemsetAsync(m->status.p, 0, 16, s));
    TrainArgs ta = train_args(m, d_features, d_tau, n, tp->sigma);
    ta.wait_ns = wait_ns;
    ta.stall = stall;
    // reduced mod n: the kernel's product of two factors below n cannot wrap
    ta.perm_mul = mul % (unsigned long long)n;
    ta.step = m->step.as<const int>();
    ta.batch = tp->batch;
    ta.sequential = 0;
    AdamArgs aa{};
    aa.partial = m->partial.as<const float>();
    aa.nparts = ctas;
    aa.inv_batch = 1.f / (float)tp->batch;
    aa.params = m->params.as<float>();
    aa.w16 = m->w16.as<__half>();
    aa.m = m->m.as<float>();
    aa.v = m->v.as<float>();
    aa.lr = tp->lr;
    aa.beta1 = tp->beta1;
    aa.beta2 = tp->beta2;
    aa.eps = tp->eps;
    aa.step = m->step.as<int>();
    aa.ticket = m->ticket.as<unsigned>();
    aa.loss_out = m->loss.as<float>();
    aa.loss_slot_by_step = 1;
    aa.loss_base = m->host_step;
    aa.status = m->status.as<const unsigned long long>();
    mlp_frozen_range(m->layers, aa.frozen_lo, aa.frozen_hi);
    // the optimiser fused into the training launch when every CTA of the
    // batch can be resident at once (its grid barrier: status word 1)
    const int resident = mlp_train_resident_ctas();
    CG_CHECK(resident > 0, CG_ERR_CUDA, "cg_mlp_train: cannot size the training kernel");
    const bool fused = !tp->separate_adam && ctas <= resident;
    if (fused) {
        ta.grid_bar = reinterpret_cast<unsigned*>(m->status.as<unsigned long long>() + 1);
        ta.adam = aa;
    }
    const int per_step = fused ? 1 : 2;
    auto one_step = [&]() -> cudaError_t {
        cudaError_t e = launch_mlp_train(ta, ctas, s);
        if (e == cudaSuccess && !fused) e = launch_mlp_adam(aa, s);
        return e;
    };
    // one eager step sets the kernels' shared-memory attributes before capture
    cudaError_t e = one_step();
    if (e != cudaSuccess) return fail(CG_ERR_CUDA, "cg_mlp_train: %s", cudaGetErrorString(e));
    ctx->launches += per_step;
    int done = 1;
    const int G = 50;
    if (tp->steps - done >= G) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        CG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < G && e == cudaSuccess; ++i) e = one_step();
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) {
            // not capturable here: the steps run as direct launches
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = nullptr;
            graph = nullptr;
            (void)cudaGetLastError();
            e = cudaSuccess;
        }
        while (exec && e == cudaSuccess && tp->steps - done >= G) {
            e = cudaGraphLaunch(exec, s);
            done += G;
            ctx->launches += (uint64_t)per_step * G;
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(CG_ERR_CUDA, "cg_mlp_train: %s", cudaGetErrorString(e));
    }
    for (; done < tp->steps; ++done) {
        e = one_step();
        if (e != cudaSuccess) return fail(CG_ERR_CUDA, "cg_mlp_train: %s", cudaGetErrorString(e));
        ctx->launches += per_step;
    }
    if (loss_per_step)
        CG_CUDA(cudaMemcpyAsync(loss_per_step, m->loss.p, (size_t)tp->steps * 4,
                                cudaMemcpyDeviceToHost, s));
    int step = 0;
    CG_CUDA(cudaMemcpyAsync(&step, m->step.p, 4, cudaMemcpyDeviceToHost, s));
    // the trained biases and output row for the renderer's constants
    std::vector<float> tail(MLP_NPARAM - MLP_B1);
    CG_CUDA(cudaMemcpyAsync(tail.data(), m->params.as<float>() + MLP_B1, tail.size() * 4,
                            cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    const int done_steps = step - m->host_step;
    m->host_step = step;
    const float* t = tail.data();  // flat layout from MLP_B1 on
    set_consts(m, t, t + (MLP_B2 - MLP_B1), t + (MLP_B3 - MLP_B1), t + (MLP_W4 - MLP_B1),
               t[MLP_B4 - MLP_B1]);
    cg_status st = train_status(m, "cg_mlp_train");
    if (st != CG_OK && loss_per_step)
        for (int i = done_steps < 0 ? 0 : done_steps; i < tp->steps; ++i)
            loss_per_step[i] = std::nanf("");  // steps that made no update
    return st;
}

extern "C" cg_status cg_mlp_get_params(const cg_mlp* m, float* params, float* adam_m,
                                       float* adam_v, int* step) {
    CG_CHECK(m && params, CG_ERR_INVALID_ARGUMENT, "cg_mlp_get_params: null pointer");
    CG_CUDA(cudaSetDevice(m->ctx->device));
    CG_CUDA(cudaStreamSynchronize(m->ctx->stream));
    CG_CUDA(cudaMemcpy(params, m->params.p, MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    if (adam_m) CG_CUDA(cudaMemcpy(adam_m, m->m.p, MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    if (adam_v) CG_CUDA(cudaMemcpy(adam_v, m->v.p, MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    if (step) CG_CUDA(cudaMemcpy(step, m->step.p, 4, cudaMemcpyDeviceToHost));
    return CG_OK;
}

extern "C" cg_status cg_mlp_set_params(cg_mlp* m, const float* params, const float* adam_m,
                                       const float* adam_v, int step) {
    CG_CHECK(m && params, CG_ERR_INVALID_ARGUMENT, "cg_mlp_set_params: null pointer");
    CG_CHECK(step >= 0, CG_ERR_OUT_OF_RANGE, "cg_mlp_set_params: step < 0");
    for (int i = 0; i < MLP_NPARAM; ++i)
        CG_CHECK(std::isfinite(params[i]), CG_ERR_INVALID_ARGUMENT,
                 "cg_mlp_set_params: non-finite parameter %d", i);
    CG_CUDA(cudaSetDevice(m->ctx->device));
    CG_CUDA(cudaStreamSynchronize(m->ctx->stream));
    cg_status st = upload_params(m, params);
    if (st != CG_OK) return st;
    // moments (zero when not given; zero for the unused layers either way)
    for (int k = 0; k < 2; ++k) {
        const float* src = k == 0 ? adam_m : adam_v;
        std::vector<float> h(MLP_NPARAM, 0.f);
        if (src) h.assign(src, src + MLP_NPARAM);
        zero_frozen(m->layers, h.data());
        CG_CUDA(cudaMemcpy((k == 0 ? m->m : m->v).p, h.data(), MLP_NPARAM * 4,
                           cudaMemcpyHostToDevice));
    }
    CG_CUDA(cudaMemcpy(m->step.p, &step, 4, cudaMemcpyHostToDevice));
    m->host_step = step;
    return CG_OK;
}

// ---- checkpoint: "CGMLPCK1", u32 version, u32 nparam, u32 nin, u32 nhidden,
// [version 2: u32 hidden layers], i32 step, cg_mlp_config, f32 params/m/v
// [nparam], u32 CRC32 of all before.  Version 1 files (three hidden layers,
// no layer count) still load.
static const char kMagic[8] = {'C', 'G', 'M', 'L', 'P', 'C', 'K', '1'};
static const uint32_t kVersion = 2;

extern "C" cg_status cg_mlp_save(const cg_mlp* m, const char* path) {
    CG_CHECK(m && path, CG_ERR_INVALID_ARGUMENT, "cg_mlp_save: null pointer");
    std::vector<float> p(MLP_NPARAM), mm(MLP_NPARAM), vv(MLP_NPARAM);
    int step = 0;
    cg_status st = cg_mlp_get_params(m, p.data(), mm.data(), vv.data(), &step);
    if (st != CG_OK) return st;
    std::vector<uint8_t> buf;
    auto put = [&](const void* d, size_t n) {
        const uint8_t* b = reinterpret_cast<const uint8_t*>(d);
        buf.insert(buf.end(), b, b + n);
    };
    uint32_t hdr[5] = {kVersion, MLP_NPARAM, MLP_IN, MLP_H, (uint32_t)m->layers};
    put(kMagic, 8);
    put(hdr, sizeof(hdr));
    put(&step, 4);
    put(&m->cfg, sizeof(cg_mlp_config));
    put(p.data(), MLP_NPARAM * 4);
    put(mm.data(), MLP_NPARAM * 4);
    put(vv.data(), MLP_NPARAM * 4);
    uint32_t crc = crc32_update(0, buf.data(), buf.size());
    put(&crc, 4);
    FILE* f = fopen(path, "wb");
    CG_CHECK(f, CG_ERR_IO, "cg_mlp_save: cannot open %s", path);
    size_t w = fwrite(buf.data(), 1, buf.size(), f);
    int c = fclose(f);
    CG_CHECK(w == buf.size() && c == 0, CG_ERR_IO, "cg_mlp_save: write failed for %s", path);
    return CG_OK;
}

extern "C" cg_status cg_mlp_load(cg_context* ctx, const char* path, cg_mlp** out) {
    CG_CHECK(ctx && path && out, CG_ERR_INVALID_ARGUMENT, "cg_mlp_load: null pointer");
    *out = nullptr;
    FILE* f = fopen(path, "rb");
    CG_CHECK(f, CG_ERR_IO, "cg_mlp_load: cannot open %s", path);
    std::vector<uint8_t> buf;
    uint8_t tmp[65536];
    size_t r;
    while ((r = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    fclose(f);
    CG_CHECK(buf.size() >= 12 && memcmp(buf.data(), kMagic, 8) == 0, CG_ERR_BAD_CHECKPOINT,
             "cg_mlp_load: bad magic");
    uint32_t version;
    memcpy(&version, buf.data() + 8, 4);
    CG_CHECK(version == 1 || version == 2, CG_ERR_BAD_CHECKPOINT,
             "cg_mlp_load: unknown version %u", version);
    const size_t hdr_words = version == 1 ? 4 : 5;
    const size_t expect =
        8 + 4 * hdr_words + 4 + sizeof(cg_mlp_config) + 3 * MLP_NPARAM * 4 + 4;
    CG_CHECK(buf.size() == expect, CG_ERR_BAD_CHECKPOINT,
             "cg_mlp_load: %s has %zu bytes, expected %zu", path, buf.size(), expect);
    uint32_t hdr[5] = {0, 0, 0, 0, 3};  // version 1: three hidden layers
    memcpy(hdr, buf.data() + 8, 4 * hdr_words);
    CG_CHECK(hdr[1] == MLP_NPARAM && hdr[2] == MLP_IN && hdr[3] == MLP_H && hdr[4] >= 1 &&
                 hdr[4] <= MLP_MAX_LAYERS,
             CG_ERR_BAD_CHECKPOINT, "cg_mlp_load: shape mismatch");
    uint32_t crc;
    memcpy(&crc, buf.data() + buf.size() - 4, 4);
    CG_CHECK(crc32_update(0, buf.data(), buf.size() - 4) == crc, CG_ERR_BAD_CHECKPOINT,
             "cg_mlp_load: CRC mismatch");
    size_t off = 8 + 4 * hdr_words;
    int step;
    memcpy(&step, buf.data() + off, 4);
    off += 4;
    cg_mlp_config cfg;
    memcpy(&cfg, buf.data() + off, sizeof(cfg));
    off += sizeof(cfg);
    std::vector<float> p(MLP_NPARAM), mm(MLP_NPARAM), vv(MLP_NPARAM);
    memcpy(p.data(), buf.data() + off, MLP_NPARAM * 4);
    off += MLP_NPARAM * 4;
    memcpy(mm.data(), buf.data() + off, MLP_NPARAM * 4);
    off += MLP_NPARAM * 4;
    memcpy(vv.data(), buf.data() + off, MLP_NPARAM * 4);
    cg_mlp* m = nullptr;
    cg_status st = cg_mlp_create_layers(ctx, 0, (int)hdr[4], &m);
    if (st != CG_OK) return st;
    st = cg_mlp_configure(m, &cfg);
    if (st == CG_OK) st = cg_mlp_set_params(m, p.data(), mm.data(), vv.data(), step);
    if (st != CG_OK) {
        cg_mlp_destroy(m);
        return st == CG_ERR_INVALID_ARGUMENT ? fail(CG_ERR_BAD_CHECKPOINT, "cg_mlp_load: %s",
                                                     cg_last_error())
                                             : st;
    }
    *out = m;
    return CG_OK;
}
