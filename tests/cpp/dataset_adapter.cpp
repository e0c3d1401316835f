// Drives fluidmarch::Dataset and fluidmarch::RayMarcher (include/fluidmarch.hpp)
// the way the reference's renderer plays a dataset: the series is loaded at
// construction, then every frame is marched in order (autoplay).  Written by
// and compared in tests/test_gpu_cpp_adapter.py.
//   argv[1] series prefix (files prefix + i + ".bgeo")
//   argv[2] camera and settings: int32 W, H, max_steps; float radius, step, iso;
//           float camera[16+16+16+3]; float depth[W*H] (the ray-start depth, shared by all frames)
//   argv[3] output: int32 frames, int64 max_particles, then per frame float positions[4*W*H]
//   argv[4] (optional) "cube": also run Dataset::makeCube and print its particle count
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fluidmarch.hpp"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    int hdr[3];
    float par[3];
    fm_camera cam{};
    if (std::fread(hdr, 4, 3, f) != 3 || std::fread(par, 4, 3, f) != 3) return 4;
    if (std::fread(cam.view, 4, 16, f) != 16 || std::fread(cam.proj, 4, 16, f) != 16 ||
        std::fread(cam.inv_proj_view, 4, 16, f) != 16 || std::fread(cam.position, 4, 3, f) != 3)
        return 4;
    cam.width = hdr[0];
    cam.height = hdr[1];
    const size_t npx = (size_t)cam.width * cam.height;
    std::vector<float> depth(npx);
    if (std::fread(depth.data(), 4, npx, f) != npx) return 4;
    std::fclose(f);
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 6;
    try {
        fluidmarch::RayMarcher marcher(0);
        fluidmarch::Dataset dataset(marcher.context(), argv[1], ".bgeo", par[0], 2.0f);
        if (!dataset.Loaded) {
            std::fprintf(stderr, "dataset: %s\n", dataset.LastError().c_str());
            return 7;
        }
        const int32_t frames = (int32_t)dataset.Frames.size();
        const int64_t maxp = (int64_t)dataset.MaxParticles;
        std::fwrite(&frames, 4, 1, o);
        std::fwrite(&maxp, 8, 1, o);
        fluidmarch::VisualizationSettings s;
        s.EnableAnisotropy = false;  // the isotropic march, compared with the oracle's
        s.MaxSteps = hdr[2];
        s.StepSize = par[1];
        s.IsoDensity = par[2];
        s.SkipMode = FM_SKIP_OFF;
        std::vector<float> pos(4 * npx), nrm(4 * npx), z(npx);
        for (s.Frame = 0; s.Frame < frames; ++s.Frame) {  // autoplay: Frame++ once a march finished
            z = depth;
            marcher.Prepare(s, cam, *dataset.Frames[s.Frame], pos.data(), nrm.data(), z.data());
            marcher.Start();
            while (!marcher.IsDone()) {
            }
            std::fwrite(pos.data(), 4, pos.size(), o);
        }
        marcher.Exit();
        if (argc > 4 && std::strcmp(argv[4], "cube") == 0) {
            fluidmarch::Dataset cube;
            fluidmarch::Dataset::makeCube(marcher.context(), cube, 0.5f, 1000, 0.1f, 2.0f, 7);
            fm_grid_info g{};
            fm_scene_grid(cube.Frames[0]->handle(), &g);
            std::printf("cube %llu %zu %d\n", (unsigned long long)g.n_particles, cube.MaxParticles, (int)cube.Loaded);
        }
    } catch (const fluidmarch::Error& e) {
        std::fprintf(stderr, "fluidmarch error %d: %s\n", e.code, e.what());
        return 5;
    }
    std::fclose(o);
    return 0;
}
