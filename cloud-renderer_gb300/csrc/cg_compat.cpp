// cg_compat.cpp -- host side of the compat render (cg_render_compat): the
// reference's billboard image formation, ConeTraceShader::coneTrace
// (ConeTraceShader.cpp:15-82).  Kernels in k_compat.cu.
#include <cmath>
#include <cstring>
#include <vector>

#include "cg_host_util.h"

namespace {

constexpr int NOISE_N = 32;

uint64_t splitmix_next(uint64_t& st) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// floor(128 |g| / sqrt(S)) capped at 127, with the sign of g: the largest
// c >= 0 with c^2 S <= 16384 g^2, found exactly in integers.
int snorm_of(int g, int64_t S) {
    if (S == 0) return 0;
    const int64_t G2 = (int64_t)16384 * g * g;
    int c = (int)std::floor(std::sqrt((double)G2 / (double)S));
    while (c > 0 && (int64_t)c * c * S > G2) --c;
    while ((int64_t)(c + 1) * (c + 1) * S <= G2) ++c;
    if (c > 127) c = 127;
    return g < 0 ? -c : c;
}

// initNoiseMap (ConeTraceShader.cpp:127-159) from a seeded stream: alpha a
// uniform in [-128, 127]; RGB the normalised "gradient" with the reference's
// operator precedence, g_x = d(x+1) - d(x-1) / 0.5 with d = a / 128 and
// wrapped neighbours (integer G = a(x+1) - 2 a(x-1)), stored as trunc(128 n)
// (0 where G = 0); decoded as GL_RGBA8_SNORM, max(c / 127, -1).
void noise_map(uint32_t seed, float* out) {
    std::vector<int8_t> a((size_t)NOISE_N * NOISE_N * NOISE_N);
    uint64_t st = (uint64_t)seed * 0x2545F4914F6CDD1DULL + 0x632BE59BD9B4E019ULL;
    for (auto& v : a) v = (int8_t)((int)(splitmix_next(st) >> 56) - 128);
    auto at = [&](int x, int y, int z) {
        x = (x % NOISE_N + NOISE_N) % NOISE_N;
        y = (y % NOISE_N + NOISE_N) % NOISE_N;
        z = (z % NOISE_N + NOISE_N) % NOISE_N;
        return (int)a[(size_t)x + (size_t)y * NOISE_N + (size_t)z * NOISE_N * NOISE_N];
    };
    for (int z = 0; z < NOISE_N; ++z)
        for (int y = 0; y < NOISE_N; ++y)
            for (int x = 0; x < NOISE_N; ++x) {
                const int g[3] = {at(x + 1, y, z) - 2 * at(x - 1, y, z),
                                  at(x, y + 1, z) - 2 * at(x, y - 1, z),
                                  at(x, y, z + 1) - 2 * at(x, y, z - 1)};
                const int64_t S = (int64_t)g[0] * g[0] + (int64_t)g[1] * g[1] +
                                  (int64_t)g[2] * g[2];
                float* o = out + 4 * ((size_t)x + (size_t)y * NOISE_N + (size_t)z * NOISE_N * NOISE_N);
                for (int k = 0; k < 3; ++k) o[k] = (float)snorm_of(g[k], S) / 127.0f;
                const float av = (float)at(x, y, z) / 127.0f;
                o[3] = av < -1.0f ? -1.0f : av;
            }
}

cg_status check_compat(const cg_compat_params* p) {
    CG_CHECK(p->num_octaves >= 0 && p->num_octaves <= 16, CG_ERR_OUT_OF_RANGE,
             "compat params: num_octaves %d not in [0, 16]", p->num_octaves);
    CG_CHECK(p->min_noise_steps >= 2 && p->max_noise_steps >= p->min_noise_steps &&
                 p->max_noise_steps <= 4096,
             CG_ERR_OUT_OF_RANGE,
             "compat params: need 2 <= min_noise_steps <= max_noise_steps <= 4096");
    CG_CHECK(p->vct_steps >= 0 && p->vct_steps <= CG_MAX_SUN_STEPS, CG_ERR_OUT_OF_RANGE,
             "compat params: vct_steps %d not in [0, %d]", p->vct_steps, CG_MAX_SUN_STEPS);
    const float vals[] = {p->step_size, p->noise_opacity, p->freq_step, p->pers_step,
                          p->adjust_size, p->min_noise_color, p->noise_color_scale,
                          p->octave_offsets[0], p->octave_offsets[1], p->octave_offsets[2],
                          p->vct_cone_angle, p->vct_cone_initial_height, p->vct_lod_offset,
                          p->vct_down_scaling, p->clear_color[0], p->clear_color[1],
                          p->clear_color[2], p->clear_color[3], p->near_plane,
                          p->transmittance_cutoff};
    for (float v : vals)
        CG_CHECK(std::isfinite(v), CG_ERR_INVALID_ARGUMENT, "compat params: non-finite value");
    CG_CHECK(p->step_size > 0.f && p->adjust_size > 0.f, CG_ERR_INVALID_ARGUMENT,
             "compat params: step_size and adjust_size must be > 0");
    CG_CHECK(p->vct_cone_angle >= 0.f && p->vct_cone_angle < 3.f, CG_ERR_OUT_OF_RANGE,
             "compat params: vct_cone_angle not in [0, 3)");
    CG_CHECK(p->vct_cone_initial_height >= 0.f && p->vct_down_scaling > 0.f,
             CG_ERR_INVALID_ARGUMENT,
             "compat params: vct_cone_initial_height >= 0 and vct_down_scaling > 0 required");
    CG_CHECK(p->near_plane > 0.f && p->near_plane < 2500.f, CG_ERR_OUT_OF_RANGE,
             "compat params: near_plane not in (0, 2500)");
    CG_CHECK(p->transmittance_cutoff >= 0.f && p->transmittance_cutoff < 1.f,
             CG_ERR_OUT_OF_RANGE, "compat params: transmittance_cutoff not in [0, 1)");
    return CG_OK;
}

}  // namespace

extern "C" void cg_compat_params_default(cg_compat_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->show_quad = 0;
    p->do_noise = 1;
    p->do_cone_trace = 1;
    p->step_size = 0.01f;
    p->noise_opacity = 4.0f;
    p->num_octaves = 4;
    p->freq_step = 3.0f;
    p->pers_step = 0.5f;
    p->adjust_size = 40.0f;
    p->min_noise_steps = 2;
    p->max_noise_steps = 8;
    p->min_noise_color = 0.2f;
    p->noise_color_scale = 0.45f;
    p->noise_seed = 1;
    p->vct_steps = 16;
    p->vct_cone_angle = 0.9f;
    p->vct_cone_initial_height = 0.1f;
    p->vct_lod_offset = 0.0f;
    p->vct_down_scaling = 1.0f;
    p->clear_color[0] = 0.2f;
    p->clear_color[1] = 0.3f;
    p->clear_color[2] = 0.5f;
    p->clear_color[3] = 1.0f;
    p->near_plane = 0.01f;
    p->transmittance_cutoff = 1e-4f;
}

extern "C" cg_status cg_compat_noise_map(uint32_t seed, float* out) {
    CG_CHECK(out, CG_ERR_INVALID_ARGUMENT, "cg_compat_noise_map: out is NULL");
    noise_map(seed, out);
    return CG_OK;
}

extern "C" cg_status cg_render_compat(cg_context* ctx, const cg_volume* v, const cg_camera* cam,
                                      const cg_compat_params* params, float* rgba_out,
                                      int out_on_device, void* stream) {
    NvtxRange nvtx_("cg_render_compat");
    CG_CHECK(ctx && v && cam && params && rgba_out, CG_ERR_INVALID_ARGUMENT,
             "cg_render_compat: null pointer");
    CG_CHECK(v->ctx == ctx, CG_ERR_INVALID_ARGUMENT,
             "cg_render_compat: volume of another context");
    cg_status st = check_compat(params);
    if (st != CG_OK) return st;
    CG_CHECK(!params->do_cone_trace || params->show_quad || v->voxelized, CG_ERR_NOT_READY,
             "cg_render_compat: the cone trace needs a voxelized volume");
    CamDesc cd;
    st = camera_of(cam, cd);
    if (st != CG_OK) return st;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    // the noise map's green and alpha channels (the fragment program reads no other)
    if (!ctx->compat_noise_valid || ctx->compat_seed != params->noise_seed) {
        std::vector<float> rgba((size_t)NOISE_N * NOISE_N * NOISE_N * 4);
        noise_map(params->noise_seed, rgba.data());
        std::vector<float> ga(rgba.size() / 2);
        for (size_t i = 0; i < rgba.size() / 4; ++i) {
            ga[2 * i] = rgba[4 * i + 1];
            ga[2 * i + 1] = rgba[4 * i + 3];
        }
        CG_CUDA(cudaStreamSynchronize(s));
        CG_CUDA(ctx->compat_noise.ensure(ga.size() * 4));
        CG_CUDA(cudaMemcpy(ctx->compat_noise.p, ga.data(), ga.size() * 4, cudaMemcpyHostToDevice));
        ctx->compat_noise_valid = true;
        ctx->compat_seed = params->noise_seed;
    }
    const size_t pixels = (size_t)cam->width * cam->height;
    float4* out = reinterpret_cast<float4*>(rgba_out);
    if (!out_on_device) {
        CG_CUDA(ctx->image.ensure(pixels * 16));
        out = ctx->image.as<float4>();
    }
    CompatDev P;
    std::memset(&P, 0, sizeof(P));
    P.cam = cd;
    P.n = v->n;
    P.cwr = v->cwr;
    P.tiles_x = (cam->width + CG_COMPAT_TILE - 1) / CG_COMPAT_TILE;
    P.tiles_y = (cam->height + CG_COMPAT_TILE - 1) / CG_COMPAT_TILE;
    P.near_z = params->near_plane;
    P.show_quad = params->show_quad != 0;
    P.do_noise = params->do_noise != 0;
    P.do_cone = params->do_cone_trace != 0;
    P.step_size = params->step_size;
    P.noise_opacity = params->noise_opacity;
    P.octaves = params->num_octaves;
    P.freq_step = params->freq_step;
    P.pers_step = params->pers_step;
    P.inv_adjust = 1.0f / params->adjust_size;
    P.min_steps = params->min_noise_steps;
    P.max_steps = params->max_noise_steps;
    P.min_color = params->min_noise_color;
    P.color_scale = params->noise_color_scale;
    for (int a = 0; a < 3; ++a) P.off[a] = params->octave_offsets[a];
    for (int a = 0; a < 4; ++a) P.clear[a] = params->clear_color[a];
    P.cutoff = params->transmittance_cutoff;
    const double sx = v->sun_dir[0], sy = v->sun_dir[1], sz = v->sun_dir[2];
    const double sn = std::sqrt(sx * sx + sy * sy + sz * sz);
    P.sun[0] = (float)(sx / sn);
    P.sun[1] = (float)(sy / sn);
    P.sun[2] = (float)(sz / sn);
    P.noise = ctx->compat_noise.as<const float2>();
    // traceCone's schedule (conetrace_frag.glsl:64-79): the reference cone mode
    TraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.sun_steps = params->vct_steps;
    tp.cone_mode = 1;
    tp.tan_half = (float)std::tan((double)params->vct_cone_angle / 2.0);
    tp.h0 = params->vct_cone_initial_height;
    tp.lod_offset = params->vct_lod_offset;
    tp.down_scaling = params->vct_down_scaling;
    const VolDesc vd = desc_of(v);
    const ConeSchedule cs = make_cone_schedule(vd, tp);
    // tile lists: counts, scan, total (one synchronisation), fill
    const int ntiles = P.tiles_x * P.tiles_y;
    const size_t cnt_words = ((size_t)ntiles + 3) & ~(size_t)3;
    const size_t off_words = ((size_t)ntiles + 1 + 3) & ~(size_t)3;
    const size_t nb = (size_t)(v->n > 0 ? v->n : 1);
    CG_CUDA(ctx->compat_rect.ensure(nb * 16));
    CG_CUDA(ctx->compat_key.ensure(nb * 4));
    // counts | offsets | cursors (u32, 16-byte aligned regions) | 64-bit pair total
    CG_CUDA(ctx->compat_tiles.ensure((cnt_words + off_words + cnt_words) * 4 + 16));
    CG_CUDA(ctx->compat_total.ensure(16));
    Bins bins{};
    bins.nbricks = ntiles;
    bins.count = ctx->compat_tiles.as<uint32_t>();
    bins.offset = bins.count + cnt_words;
    bins.cursor = bins.offset + off_words;
    unsigned long long* pairs64 = reinterpret_cast<unsigned long long*>(bins.cursor + cnt_words);
    stage_begin(ctx, s);
    CG_CUDA(cudaMemsetAsync(bins.count, 0, cnt_words * 4, s));
    CG_CUDA(cudaMemsetAsync(pairs64, 0, 8, s));
    CG_LAUNCH(ctx, launch_compat_count(P, ctx->compat_rect.as<int4>(), ctx->compat_key.as<float>(),
                                       bins.count, pairs64, s));
    CG_LAUNCH(ctx, launch_bin_scan(bins, s));
    uint64_t* total = reinterpret_cast<uint64_t*>(ctx->compat_total.p);
    CG_CUDA(cudaMemcpyAsync(total, pairs64, 8, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    // the per-tile offsets are 32-bit
    CG_CHECK(*total < 0xFFFFFFFFull, CG_ERR_OUT_OF_RANGE,
             "cg_render_compat: %llu board-tile pairs exceed 2^32 (fewer boards or pixels)",
             (unsigned long long)*total);
    CG_CUDA(ctx->compat_list.ensure((size_t)(*total > 0 ? *total : 1) * 8));
    CG_LAUNCH(ctx, launch_compat_fill(P, ctx->compat_rect.as<const int4>(),
                                      ctx->compat_key.as<const float>(), bins.cursor,
                                      ctx->compat_list.as<unsigned long long>(), s));
    stage_mark(ctx, s, "bin");
    CG_LAUNCH(ctx, launch_compat_tiles(vd, cs, P, bins.offset,
                                       ctx->compat_list.as<unsigned long long>(), out, s));
    stage_mark(ctx, s, "tiles");
    if (!out_on_device) {
        CG_CUDA(cudaMemcpyAsync(rgba_out, out, pixels * 16, cudaMemcpyDeviceToHost, s));
        CG_CUDA(cudaStreamSynchronize(s));
    }
    return CG_OK;
}
