/*
 * cloudgb.hpp -- C++17 host mirror of the reference's classes over the C ABI
 * (cloudgb.h): CloudVolume, VoxelizeShader, ConeTraceShader, Sun, Camera, with
 * the reference's member names and meanings (CloudVolume.hpp:12-55,
 * VoxelizeShader.hpp:9-33, ConeTraceShader.hpp:10-36), so that the
 * reference's frame (main.cpp:98-140),
 *
 *     volume->update();  voxelizeShader->voxelize(volume);  coneShader->coneTrace(volume);
 *
 * keeps its shape.  Header-only; link libcloudgb.so.  Failures throw
 * cloudgb::Error carrying the cg_status and cg_last_error() (the reference
 * printed GL errors, GLSL.hpp:40-44, or exit()ed, Shader.cpp:35-36).
 *
 * What differs from the reference: the sun is a direction (cg_sun) and the
 * camera an explicit pinhole (cg_camera) passed to the calls, instead of the
 * Sun / Camera statics; coneTrace returns the image (RGBA32F, row 0 = top)
 * instead of drawing into the window; boards carry a density.
 */
#ifndef CLOUDGB_HPP
#define CLOUDGB_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cloudgb.h"

namespace cloudgb {

struct Vec2 {
    float x = 0.f, y = 0.f;
};
struct Vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
};
struct IVec3 {
    int x = 0, y = 0, z = 0;
};

class Error : public std::runtime_error {
   public:
    Error(cg_status s, const std::string& what)
        : std::runtime_error(what + ": " + cg_last_error()), status(s) {}
    cg_status status;
};

inline void check(cg_status s, const char* what) {
    if (s != CG_OK) throw Error(s, what);
}

// One context per device (the reference's GL context, Window::init).
class Context {
   public:
    explicit Context(int device = 0) { check(cg_context_create(device, &ctx_), "cg_context_create"); }
    ~Context() { cg_context_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    cg_context* handle() const { return ctx_; }
    void synchronize() { check(cg_context_synchronize(ctx_), "cg_context_synchronize"); }
    uint64_t launchCount() const { return cg_context_launch_count(ctx_); }

   private:
    cg_context* ctx_ = nullptr;
};

// A directional sun and the size of its sun-view map (the reference's
// Sun::position and position FBO, Sun.hpp:26-43, VoxelizeShader.cpp:136-167).
struct Sun {
    Vec3 direction{0.3f, 1.f, 0.2f};
    int mapWidth = 1280, mapHeight = 720;
    cg_sun c() const { return cg_sun{{direction.x, direction.y, direction.z}, mapWidth, mapHeight}; }
};

// Pinhole camera (Camera::getP / getV, Camera.cpp:59-60).
struct Camera {
    Vec3 eye{0.f, 0.f, -2.f}, target{0.f, 0.f, 0.f}, up{0.f, 1.f, 0.f};
    float fovY = 60.f;  // degrees
    int width = 256, height = 256;
    cg_camera c() const {
        return cg_camera{{eye.x, eye.y, eye.z}, {target.x, target.y, target.z},
                         {up.x, up.y, up.z}, fovY, width, height};
    }
};

// CloudVolume(int dim, vec2 bounds, vec3 position, int mips) (CloudVolume.cpp:7-55).
class CloudVolume {
   public:
    struct Billboards {
        std::vector<Vec3> positions;  // relative to `position`
        std::vector<float> scales;    // radii
        std::vector<float> densities; // per board (this build's density volume)
        int count = 0;
        Vec3 minOffset{-1.f, -1.f, -1.f}, maxOffset{1.f, 1.f, 1.f};
        float minScale = 1.f, maxScale = 1.f;
        uint64_t seed = 0;
    };

    CloudVolume(Context& ctx, int dim, Vec2 bounds, Vec3 position, int mips,
                cg_format format = CG_FORMAT_RGBA32F)
        : position(position), xBounds(bounds), yBounds(bounds), zBounds(bounds), dimension(dim),
          levels(mips), format(format) {
        const float r = bounds.y - bounds.x;
        range = Vec3{r, r, r};
        voxelSize = Vec3{r / dim, r / dim, r / dim};
        const float p[3] = {position.x, position.y, position.z};
        check(cg_volume_create(ctx.handle(), dim, bounds.x, bounds.y, p, mips, format, &vol_),
              "cg_volume_create");
    }
    ~CloudVolume() { cg_volume_destroy(vol_); }
    CloudVolume(const CloudVolume&) = delete;
    CloudVolume& operator=(const CloudVolume&) = delete;

    // CloudVolume::update (CloudVolume.cpp:84-93): upload the billboards.
    void update() { uploadBillboards(); }
    // The volume is cleared by every voxelize (CloudVolume.cpp:96-100).
    void clearGPU() {}

    // CloudVolume::addCloudBoard (CloudVolume.cpp:58-62).
    void addCloudBoard(const Vec3& pos, float scale, float density = 1.f) {
        billboards.positions.push_back(pos);
        billboards.scales.push_back(scale);
        billboards.densities.push_back(density);
        billboards.count = (int)billboards.positions.size();
    }

    // Far-to-near order by distance to `point` (CloudVolume.cpp:65-82); a stable
    // sort.  The renderer composites front to back per pixel and does not need
    // it; it only changes which board wins a sun-map depth tie.
    void sortBoards(const Vec3& point) {
        const size_t n = billboards.positions.size();
        std::vector<float> d(n);
        for (size_t i = 0; i < n; ++i) {
            const Vec3& q = billboards.positions[i];
            const float dx = position.x + q.x - point.x, dy = position.y + q.y - point.y,
                        dz = position.z + q.z - point.z;
            d[i] = std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        std::vector<size_t> order(n);
        std::iota(order.begin(), order.end(), size_t(0));
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return d[a] > d[b]; });
        Billboards s = billboards;
        for (size_t i = 0; i < n; ++i) {
            s.positions[i] = billboards.positions[order[i]];
            s.scales[i] = billboards.scales[order[i]];
            s.densities[i] = billboards.densities[order[i]];
        }
        billboards = std::move(s);
    }

    // CloudVolume::uploadBillboards (CloudVolume.cpp:139-164), fluffiness
    // multiplying the radii.
    void uploadBillboards() {
        const int n = (int)billboards.positions.size();
        if ((int)billboards.densities.size() != n) billboards.densities.assign(n, 1.f);
        billboards.count = n;
        std::vector<float> p(3 * (size_t)n);
        for (int i = 0; i < n; ++i) {
            p[3 * i] = billboards.positions[i].x;
            p[3 * i + 1] = billboards.positions[i].y;
            p[3 * i + 2] = billboards.positions[i].z;
        }
        check(cg_volume_set_billboards(vol_, p.data(), billboards.scales.data(),
                                       billboards.densities.data(), n, fluffiness),
              "cg_volume_set_billboards");
    }

    // CloudVolume::regenerateBillboards (CloudVolume.cpp:120-133): offsets
    // uniform in [minOffset, maxOffset], scales in [minScale, maxScale], drawn
    // from a SplitMix64 stream of `seed` (53-bit doubles; x, y, z of every board
    // first, then the scales) -- the same stream as the Python mirror.
    void regenerateBillboards(int count, Vec3 minOffset, Vec3 maxOffset, float minScale,
                              float maxScale, uint64_t seed = 0) {
        regenerate(billboards, count, minOffset, maxOffset, minScale, maxScale, seed);
    }
    // The generator alone (no device needed).
    static void regenerate(Billboards& b, int count, Vec3 minOffset, Vec3 maxOffset,
                           float minScale, float maxScale, uint64_t seed) {
        b.minOffset = minOffset;
        b.maxOffset = maxOffset;
        b.minScale = minScale;
        b.maxScale = maxScale;
        b.seed = seed;
        uint64_t st = seed;
        auto uni = [&]() {
            uint64_t z = (st += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            return (double)(z >> 11) * (1.0 / 9007199254740992.0);
        };
        b.positions.assign(count, Vec3{});
        b.scales.assign(count, 0.f);
        b.densities.assign(count, 1.f);
        const double lo[3] = {minOffset.x, minOffset.y, minOffset.z};
        const double hi[3] = {maxOffset.x, maxOffset.y, maxOffset.z};
        for (int i = 0; i < count; ++i) {
            double v[3];
            for (int a = 0; a < 3; ++a) v[a] = lo[a] + (hi[a] - lo[a]) * uni();
            b.positions[i] = Vec3{(float)v[0], (float)v[1], (float)v[2]};
        }
        for (int i = 0; i < count; ++i)
            b.scales[i] = (float)((double)minScale + ((double)maxScale - (double)minScale) * uni());
        b.count = count;
    }
    void resetBillboards() {
        regenerateBillboards((int)billboards.positions.size(), billboards.minOffset,
                             billboards.maxOffset, billboards.minScale, billboards.maxScale,
                             billboards.seed);
    }

    IVec3 get3DIndices(int index) const {
        const int line = dimension, slice = dimension * dimension;
        const int z = index / slice, y = (index - z * slice) / line;
        return IVec3{index - z * slice - y * line, y, z};
    }
    Vec3 reverseVoxelIndex(const IVec3& i) const {
        return Vec3{(float)i.x * range.x / dimension + xBounds.x,
                    (float)i.y * range.y / dimension + yBounds.x,
                    (float)i.z * range.z / dimension + zBounds.x};
    }
    // The reference's voxel-view statistic (VoxelShader.cpp:110-119).
    uint64_t activeVoxels() const {
        uint64_t v = 0;
        check(cg_volume_active_voxels(vol_, &v), "cg_volume_active_voxels");
        return v;
    }
    cg_volume* handle() const { return vol_; }

    Vec3 position;
    Vec2 xBounds, yBounds, zBounds;
    int dimension;
    Vec3 range, voxelSize;
    int levels;
    cg_format format;
    Billboards billboards;
    float fluffiness = 1.f;

   private:
    cg_volume* vol_ = nullptr;
};

// VoxelizeShader::voxelize(CloudVolume*) (VoxelizeShader.cpp:18-31).
class VoxelizeShader {
   public:
    Sun sun;
    void voxelize(CloudVolume* volume, void* stream = nullptr) {
        const cg_sun s = sun.c();
        check(cg_voxelize(volume->handle(), &s, stream), "cg_voxelize");
    }
};

// ConeTraceShader::coneTrace(CloudVolume*) (ConeTraceShader.cpp:15-82) with the
// public fields of ConeTraceShader.hpp:15-32 (vctConeAngle = full aperture).
class ConeTraceShader {
   public:
    ConeTraceShader() {
        cg_render_params p;
        cg_render_params_default(&p);
        viewSteps = p.view_steps;
        vctSteps = p.sun_steps;
        vctConeAngle = 2.f * p.cone_half_angle;
        vctConeInitialHeight = p.cone_initial_height;
        vctConeMinRadius = p.cone_min_radius;
        vctLodOffset = p.lod_offset;
        vctDownScaling = p.down_scaling;
        densityScale = p.density_scale;
        ambient = p.ambient;
        sunColor = Vec3{p.sun_color[0], p.sun_color[1], p.sun_color[2]};
        transmittanceCutoff = p.transmittance_cutoff;
        coneMode = p.cone_mode;
        noiseSeed = p.noise.seed;
        numOctaves = p.noise.octaves;
        noiseFrequency = p.noise.frequency;
        freqStep = p.noise.lacunarity;
        persStep = p.noise.gain;
        pipeline = p.pipeline;
        coneLanes = p.cone_lanes;
    }

    int viewSteps, vctSteps;
    float vctConeAngle, vctConeInitialHeight, vctConeMinRadius, vctLodOffset, vctDownScaling;
    float densityScale, ambient;
    Vec3 sunColor;
    float transmittanceCutoff;
    int coneMode;
    uint32_t noiseSeed;
    int numOctaves;
    float noiseFrequency, freqStep, persStep;
    Vec3 windVel{0.01f, 0.f, 0.f};  // ConeTraceShader.hpp:25
    float runTime = 0.f;            // Window::runTime (set by the caller)
    bool useMlp = false;
    const cg_mlp* mlp = nullptr;
    int pipeline;
    int coneLanes;
    Camera camera;

    cg_render_params params() const {
        cg_render_params p;
        cg_render_params_default(&p);
        p.view_steps = viewSteps;
        p.sun_steps = vctSteps;
        p.cone_half_angle = vctConeAngle / 2.f;
        p.cone_initial_height = vctConeInitialHeight;
        p.cone_min_radius = vctConeMinRadius;
        p.lod_offset = vctLodOffset;
        p.down_scaling = vctDownScaling;
        p.density_scale = densityScale;
        p.ambient = ambient;
        p.sun_color[0] = sunColor.x;
        p.sun_color[1] = sunColor.y;
        p.sun_color[2] = sunColor.z;
        p.transmittance_cutoff = transmittanceCutoff;
        p.cone_mode = coneMode;
        p.noise.seed = noiseSeed;
        p.noise.octaves = numOctaves;
        p.noise.frequency = noiseFrequency;
        p.noise.lacunarity = freqStep;
        p.noise.gain = persStep;
        p.noise.offset[0] = windVel.x * runTime;
        p.noise.offset[1] = windVel.y * runTime;
        p.noise.offset[2] = windVel.z * runTime;
        p.use_mlp = useMlp ? 1 : 0;
        p.mlp = useMlp ? mlp : nullptr;
        p.pipeline = pipeline;
        p.cone_lanes = coneLanes;
        return p;
    }

    // The camera's view of the volume: width * height * 4 floats, row 0 = top.
    std::vector<float> coneTrace(CloudVolume* volume, Context& ctx) {
        std::vector<float> img((size_t)camera.width * camera.height * 4);
        coneTrace(volume, ctx, img.data(), false, nullptr);
        return img;
    }
    // Into a host buffer (synchronous) or a device buffer (asynchronous on stream).
    void coneTrace(CloudVolume* volume, Context& ctx, float* out, bool on_device, void* stream) {
        const cg_render_params p = params();
        const cg_camera c = camera.c();
        check(cg_render(ctx.handle(), volume->handle(), &c, &p, out, on_device ? 1 : 0, stream),
              "cg_render");
    }
};

}  // namespace cloudgb

#endif  // CLOUDGB_HPP
