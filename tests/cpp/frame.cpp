// frame.cpp -- the reference's frame through the C++ mirror (cloudgb.hpp):
//   volume->update(); voxelizeShader->voxelize(volume); coneShader->coneTrace(volume);
// Built and run by tests/test_cpp_api.py.
//   frame regen <out> <count> <seed>   boards of regenerateBillboards (host only)
//   frame render <in> <out>            one frame of the scene in <in>
//   frame version                      the library's ABI version (host only)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cloudgb.hpp"

using namespace cloudgb;

template <class T>
static void get(FILE* f, T* p, size_t n) {
    if (fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input file");
}

int main(int argc, char** argv) {
    try {
        if (argc >= 2 && !strcmp(argv[1], "version")) {
            printf("%d\n", cg_abi_version());
            return 0;
        }
        if (argc == 5 && !strcmp(argv[1], "regen")) {
            CloudVolume::Billboards b;
            CloudVolume::regenerate(b, atoi(argv[3]), Vec3{-2.5f, -2.5f, -2.5f},
                                    Vec3{2.5f, 2.5f, 2.5f}, 1.f, 2.5f,
                                    (uint64_t)strtoull(argv[4], nullptr, 10));
            FILE* o = fopen(argv[2], "wb");
            if (!o) return 2;
            for (const Vec3& p : b.positions) fwrite(&p, sizeof(float), 3, o);
            fwrite(b.scales.data(), sizeof(float), b.scales.size(), o);
            fclose(o);
            return 0;
        }
        if (argc == 4 && !strcmp(argv[1], "render")) {
            FILE* f = fopen(argv[2], "rb");
            if (!f) return 2;
            int32_t hdr[8];  // n, dim, mips, mapW, mapH, width, height, octaves
            get(f, hdr, 8);
            float geo[13];   // bounds (2), position (3), sun (3), eye (3), fov, fluffiness
            get(f, geo, 13);
            float tgt[3];
            get(f, tgt, 3);
            int32_t ip[3];   // viewSteps, vctSteps, noiseSeed
            get(f, ip, 3);
            float fp[12];    // vctConeAngle, vctConeInitialHeight, vctConeMinRadius,
                             // densityScale, ambient, noiseFrequency, freqStep, persStep,
                             // runTime, windVel (3)
            get(f, fp, 12);
            const int n = hdr[0];
            std::vector<float> pos(3 * (size_t)n), sc(n), den(n);
            get(f, pos.data(), pos.size());
            get(f, sc.data(), sc.size());
            get(f, den.data(), den.size());
            fclose(f);

            Context ctx(0);
            CloudVolume volume(ctx, hdr[1], Vec2{geo[0], geo[1]}, Vec3{geo[2], geo[3], geo[4]},
                               hdr[2]);
            for (int i = 0; i < n; ++i)
                volume.addCloudBoard(Vec3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, sc[i],
                                     den[i]);
            volume.fluffiness = geo[12];
            VoxelizeShader voxelizer;
            voxelizer.sun = Sun{Vec3{geo[5], geo[6], geo[7]}, hdr[3], hdr[4]};
            ConeTraceShader cone;
            cone.camera.eye = Vec3{geo[8], geo[9], geo[10]};
            cone.camera.target = Vec3{tgt[0], tgt[1], tgt[2]};
            cone.camera.fovY = geo[11];
            cone.camera.width = hdr[5];
            cone.camera.height = hdr[6];
            cone.viewSteps = ip[0];
            cone.vctSteps = ip[1];
            cone.noiseSeed = (uint32_t)ip[2];
            cone.numOctaves = hdr[7];
            cone.vctConeAngle = fp[0];
            cone.vctConeInitialHeight = fp[1];
            cone.vctConeMinRadius = fp[2];
            cone.densityScale = fp[3];
            cone.ambient = fp[4];
            cone.noiseFrequency = fp[5];
            cone.freqStep = fp[6];
            cone.persStep = fp[7];
            cone.runTime = fp[8];
            cone.windVel = Vec3{fp[9], fp[10], fp[11]};

            // the reference's frame (main.cpp:98-140)
            volume.update();
            voxelizer.voxelize(&volume);
            std::vector<float> img = cone.coneTrace(&volume, ctx);

            FILE* o = fopen(argv[3], "wb");
            if (!o) return 2;
            fwrite(img.data(), sizeof(float), img.size(), o);
            fclose(o);
            printf("active voxels %llu\n", (unsigned long long)volume.activeVoxels());
            return 0;
        }
        fprintf(stderr, "usage: frame version | regen <out> <count> <seed> | render <in> <out>\n");
        return 1;
    } catch (const Error& e) {
        fprintf(stderr, "cloudgb error %d: %s\n", (int)e.status, e.what());
        return 3;
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        return 4;
    }
}
